"""ctypes binding of liblpm_bve.so (the C ABI declared in include/lpm_bve*.h).

The shared library is built in-tree by ``lpmkokkos_gb300._build.build()``.  Loading
fails loudly if it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

LPM_OK = 0
LPM_ERR_INVALID_ARGUMENT = -1
LPM_ERR_CUDA = -2
LPM_ERR_OUT_OF_MEMORY = -3
LPM_ERR_NOT_SUPPORTED = -4
LPM_ERR_ADMISSION = -5
LPM_ERR_STATE = -6
LPM_ERR_TIMEOUT = -7
LPM_ERR_INTERNAL = -8

FP64 = 0
FP32C = 1 << 0
COLLOCATED = 1 << 1
PSI = 1 << 2
NO_VELOCITY = 1 << 3
RK4_FIX_QUIRK = 1 << 4
RENORM = 1 << 5
SKIP_MASKED_TARGETS = 1 << 6
NO_GRAPH = 1 << 7
NO_SORT = 1 << 8
MESH_TARGETS = 1 << 9
RCP_APPROX = 1 << 10
TREECODE = 1 << 11
NO_SYMMETRIC = 1 << 12

SEED_ICOS_TRI = 0
SEED_CUBED = 1

c_i64 = ctypes.c_int64
c_dp = ctypes.POINTER(ctypes.c_double)


class Opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("autotune", ctypes.c_int), ("verbose", ctypes.c_int)]


class Points(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("n", c_i64), ("stride_i", c_i64), ("stride_c", c_i64)]


class Sources(ctypes.Structure):
    _fields_ = [("pts", Points), ("zeta", ctypes.c_void_p), ("area", ctypes.c_void_p), ("mask", ctypes.c_void_p)]


class State(ctypes.Structure):
    _fields_ = [
        ("nverts", c_i64), ("nfaces", c_i64),
        ("vx", ctypes.c_void_p), ("vx_stride_i", c_i64), ("vx_stride_c", c_i64),
        ("vzeta", ctypes.c_void_p),
        ("vvel", ctypes.c_void_p), ("vvel_stride_i", c_i64), ("vvel_stride_c", c_i64),
        ("fx", ctypes.c_void_p), ("fx_stride_i", c_i64), ("fx_stride_c", c_i64),
        ("fzeta", ctypes.c_void_p),
        ("fvel", ctypes.c_void_p), ("fvel_stride_i", c_i64), ("fvel_stride_c", c_i64),
        ("farea", ctypes.c_void_p), ("fmask", ctypes.c_void_p),
    ]


class ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t), ("max_active", ctypes.c_int),
                ("flags", ctypes.c_uint), ("eps", ctypes.c_double), ("host_ic", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_int), ("level", ctypes.c_int), ("ic_seed", ctypes.c_uint64),
                ("n_gaussians", ctypes.c_int), ("gauss_width", ctypes.c_double), ("dt", ctypes.c_double),
                ("omega", ctypes.c_double), ("nsteps", ctypes.c_int)]


class ServerCounters(ctypes.Structure):
    _fields_ = [("submitted", c_i64), ("completed", c_i64), ("failed", c_i64), ("cancelled", c_i64),
                ("running", c_i64), ("queued", c_i64), ("steps_run", c_i64), ("solve_steps", c_i64),
                ("pairs", ctypes.c_double), ("busy_s", ctypes.c_double), ("reserved_bytes", ctypes.c_size_t),
                ("budget_bytes", ctypes.c_size_t), ("max_running_seen", ctypes.c_int),
                ("tree_equiv_pairs", ctypes.c_double)]


NORMS_ABS_LINF = 1 << 0

REQ_QUEUED, REQ_PREPARING, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, -1, -2

_lib = None


class LpmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"lpm_bve error {code}: {msg}")
        self.code = code


def _declare(L):
    vp = ctypes.c_void_p
    L.lpm_bve_ctx_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Opts)]
    L.lpm_bve_ctx_destroy.argtypes = [vp]
    L.lpm_bve_last_error.argtypes = [vp]
    L.lpm_bve_last_error.restype = ctypes.c_char_p
    L.lpm_bve_plan_invalidate.argtypes = [vp]
    L.lpm_bve_ctx_set_timing.argtypes = [vp, ctypes.c_int]
    L.lpm_bve_ctx_timing.argtypes = [vp, c_dp, ctypes.POINTER(c_i64), ctypes.c_int]
    ip = ctypes.POINTER(ctypes.c_int)
    L.lpm_bve_ctx_shapes.argtypes = [ip, ip, ip, ip, ctypes.c_int]
    L.lpm_bve_ctx_set_shape.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.lpm_bve_velocity.argtypes = [vp, ctypes.POINTER(Points), ctypes.POINTER(Sources), vp, c_i64, c_i64, vp,
                                   ctypes.c_uint, ctypes.c_double, vp]
    L.lpm_bve_rk4_increments.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp, vp]
    L.lpm_bve_rk4_step.argtypes = [vp, ctypes.POINTER(State), ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_uint, ctypes.c_double, vp]
    L.lpm_bve_ensemble_create.argtypes = [vp, ctypes.POINTER(State), ctypes.c_int, ctypes.c_uint, ctypes.c_double,
                                          vp, ctypes.POINTER(vp)]
    L.lpm_bve_ensemble_step.argtypes = [vp, c_dp, c_dp, ctypes.c_int, vp]
    L.lpm_bve_ensemble_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(c_i64),
                                        ctypes.POINTER(ctypes.c_size_t)]
    L.lpm_bve_ensemble_destroy.argtypes = [vp]
    L.lpm_mesh_counts.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64),
                                  ctypes.POINTER(c_i64)]
    L.lpm_mesh_build.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, vp, vp]
    for n in ("lpm_ic_rh54", "lpm_ic_rh54_velocity", "lpm_ic_solid_body"):
        getattr(L, n).argtypes = [vp, c_i64, vp]
    L.lpm_ic_gaussians_add.argtypes = [vp, c_i64, vp, vp, ctypes.c_int, ctypes.c_double, vp]
    L.lpm_probe_fp32_fma.argtypes = [ctypes.c_int, ctypes.c_int, c_dp, c_dp]
    L.lpm_probe_fp32_fma2.argtypes = [ctypes.c_int, ctypes.c_int, c_dp, c_dp]
    L.lpm_ic_gaussian_params.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, vp]
    L.lpm_ic_rh54_gaussians_device.argtypes = [vp, c_i64, c_i64, c_i64, vp, vp, ctypes.c_int, ctypes.c_double, vp,
                                               vp]
    L.lpm_sphere_tangency.argtypes = [vp, c_i64, c_i64, vp, c_i64, c_i64, c_i64, vp, vp]
    L.lpm_bve_ctx_set_treecode.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double]
    L.lpm_bve_ctx_set_symmetric.argtypes = [vp, c_i64]
    L.lpm_bve_ctx_tree_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(c_i64),
                                         ctypes.POINTER(c_i64), c_dp, c_dp, c_dp, c_dp]
    L.lpm_octree_build.argtypes = [vp, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp), vp]
    c_ip = ctypes.POINTER(ctypes.c_int32)
    L.lpm_octree_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), c_ip,
                                  c_ip, c_dp]
    L.lpm_octree_arrays.argtypes = [vp] + [ctypes.POINTER(vp)] * 8
    L.lpm_octree_destroy.argtypes = [vp]
    L.lpm_errnorms.argtypes = [vp, vp, c_i64, c_i64, vp, c_i64, c_i64, vp, vp, c_i64, ctypes.c_int, ctypes.c_uint,
                               c_dp, vp]
    L.lpm_bve_server_create.argtypes = [ctypes.POINTER(ServerOpts), ctypes.POINTER(vp)]
    L.lpm_bve_server_estimate.argtypes = [ctypes.POINTER(ServerOpts), ctypes.POINTER(Request),
                                          ctypes.POINTER(ctypes.c_size_t)]
    L.lpm_bve_server_submit.argtypes = [vp, ctypes.POINTER(Request), ctypes.POINTER(c_i64)]
    L.lpm_bve_server_wait.argtypes = [vp, c_i64, ctypes.c_double]
    L.lpm_bve_server_status.argtypes = [vp, c_i64, ctypes.POINTER(ctypes.c_int)]
    L.lpm_bve_server_cancel.argtypes = [vp, c_i64]
    L.lpm_bve_server_result.argtypes = [vp, c_i64, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), vp, vp, vp, vp, vp,
                                        vp]
    L.lpm_bve_server_release.argtypes = [vp, c_i64]
    L.lpm_bve_server_snapshot.argtypes = [vp, c_i64, ctypes.c_char_p]
    L.lpm_bve_snapshot_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(State), ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
    L.lpm_bve_snapshot_info.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), c_dp, c_dp, c_dp]
    L.lpm_bve_snapshot_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(State), c_dp, vp]
    L.lpm_bve_vtk_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(State), ctypes.c_int, ctypes.c_int, vp]
    L.lpm_mesh_face_verts.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_int)]
    L.lpm_bve_server_timing.argtypes = [vp, c_i64, c_dp, c_dp, c_dp]
    L.lpm_bve_server_latency.argtypes = [vp, c_dp, ctypes.c_int, c_dp]
    L.lpm_bve_server_stats.argtypes = [vp, ctypes.POINTER(ServerCounters)]
    L.lpm_bve_server_last_error.argtypes = [vp]
    L.lpm_bve_server_last_error.restype = ctypes.c_char_p
    L.lpm_bve_server_destroy.argtypes = [vp]


def lib(build_if_missing: bool = False):
    """The loaded native library.  Raises if it was not built (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            if not build_if_missing:
                raise RuntimeError(
                    f"native library {_build.LIB} is missing: run lpmkokkos_gb300._build.build() "
                    "(python -c 'import __graft_entry__ as g; g.build()')")
            _build.build()
        L = ctypes.CDLL(_build.LIB)
        _declare(L)
        _lib = L
    return _lib


def check(rc, ctx=None):
    if rc != LPM_OK:
        msg = lib().lpm_bve_last_error(ctx).decode() if ctx else ""
        raise LpmError(rc, msg)
    return rc
