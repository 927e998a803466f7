"""Host-side mirror of the reference's BVE interface over the C ABI.

pbosler/lpmKokkos keeps the BVE problem in ``BVESphere<Seed>`` (src/LpmBVESphere.hpp:18-80)
and steps it with ``BVERK4`` (src/LpmBVERK4.hpp:13-65).  The classes below keep those names,
members and argument meanings for Python callers; device arrays are torch tensors used as
plain device buffers, and every computation goes through liblpm_bve.so.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np
import torch

from . import _lib as L

PI = math.pi


def _vp(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else None


def _np_ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _stream(stream) -> ctypes.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _points(x: torch.Tensor) -> L.Points:
    assert x.dtype == torch.float64 and x.dim() == 2 and x.shape[1] == 3, "positions must be float64 (n, 3)"
    return L.Points(x.data_ptr() if x.numel() else None, x.shape[0], x.stride(0), x.stride(1))


def _mask_ptr(m: Optional[torch.Tensor]):
    if m is None:
        return None
    assert m.dtype in (torch.uint8, torch.bool), "mask must be uint8 or bool"
    return m.data_ptr() if m.numel() else None


# ----------------------------------------------------------------------------------------
# host mesh and initial conditions
# ----------------------------------------------------------------------------------------
def mesh_counts(seed: int, level: int):
    nv, nf, nl = L.c_i64(), L.c_i64(), L.c_i64()
    L.check(L.lib().lpm_mesh_counts(seed, level, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(nl)))
    return nv.value, nf.value, nl.value


def build_mesh(seed: int, level: int) -> dict:
    """Uniformly refined icosahedral (seed 0) or cubed-sphere (seed 1) mesh, host numpy arrays."""
    nv, nf, nl = mesh_counts(seed, level)
    vx = np.zeros((nv, 3)); fx = np.zeros((nf, 3)); fa = np.zeros(nf); fm = np.zeros(nf, dtype=np.uint8)
    L.check(L.lib().lpm_mesh_build(seed, level, _np_ptr(vx), _np_ptr(fx), _np_ptr(fa), _np_ptr(fm)))
    return dict(seed=seed, level=level, nverts=nv, nfaces=nf, nleaves=nl, vx=vx, fx=fx, farea=fa, fmask=fm)


def _map(fn, x: np.ndarray, width: int):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.shape[0], width) if width > 1 else x.shape[0])
    L.check(fn(_np_ptr(x), x.shape[0], _np_ptr(out)))
    return out


def ic_rh54(x: np.ndarray) -> np.ndarray:
    return _map(L.lib().lpm_ic_rh54, x, 1)


def rh54_velocity(x: np.ndarray) -> np.ndarray:
    return _map(L.lib().lpm_ic_rh54_velocity, x, 3)


def ic_solid_body(x: np.ndarray) -> np.ndarray:
    return _map(L.lib().lpm_ic_solid_body, x, 1)


def gaussian_params(seed: int, ng: int, amp_lo: float = -2.0, amp_hi: float = 2.0):
    c = np.zeros((ng, 3)); a = np.zeros(ng)
    L.check(L.lib().lpm_ic_gaussian_params(seed, ng, amp_lo, amp_hi, _np_ptr(c), _np_ptr(a)))
    return c, a


def ic_gaussians_add(x: np.ndarray, zeta: np.ndarray, centers, amps, width: float = 0.1) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    z = np.array(zeta, dtype=np.float64, copy=True)
    c = np.ascontiguousarray(centers, dtype=np.float64)
    a = np.ascontiguousarray(amps, dtype=np.float64)
    L.check(L.lib().lpm_ic_gaussians_add(_np_ptr(x), x.shape[0], _np_ptr(c), _np_ptr(a), a.shape[0], width,
                                         _np_ptr(z)))
    return z


def rh54_gaussians(seed: int, ng: int, width: float = 0.1) -> Callable[[np.ndarray], np.ndarray]:
    """Relative-vorticity initial condition: RH54 plus ng seeded Gaussian vortices."""
    c, a = gaussian_params(seed, ng)

    def ic(x):
        return ic_gaussians_add(x, ic_rh54(x), c, a, width) if ng > 0 else ic_rh54(x)
    ic.centers, ic.amps, ic.width = c, a, width
    return ic


def ic_rh54_gaussians_device(x: torch.Tensor, seed: int, ng: int, width: float = 0.1, stream=None) -> torch.Tensor:
    """rh54_gaussians(seed, ng, width) evaluated on the device at float64 (n, 3) device points."""
    assert x.dtype == torch.float64 and x.dim() == 2 and x.shape[1] == 3 and x.is_cuda
    c, a = gaussian_params(seed, ng)
    z = torch.empty(x.shape[0], dtype=torch.float64, device=x.device)
    L.check(L.lib().lpm_ic_rh54_gaussians_device(_vp(x), x.shape[0], x.stride(0), x.stride(1), _np_ptr(c),
                                                 _np_ptr(a), ng, width, _vp(z), _stream(stream)))
    return z


def sphere_tangency(x: torch.Tensor, u: torch.Tensor, out: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
    """u . x per point of float64 (n, 3) device arrays (SphereVelocityTangentTestFunctor,
    src/LpmSphereTestKernels.hpp:11-25); zero up to rounding for a tangent velocity field."""
    assert x.dtype == u.dtype == torch.float64 and x.is_cuda and u.is_cuda and x.shape == u.shape and x.shape[1] == 3
    if out is None:
        out = torch.empty(x.shape[0], dtype=torch.float64, device=x.device)
    L.check(L.lib().lpm_sphere_tangency(_vp(x), x.stride(0), x.stride(1), _vp(u), u.stride(0), u.stride(1),
                                        x.shape[0], _vp(out), _stream(stream)))
    return out


class _DeviceView:
    """A borrowed device array, exposed to torch through __cuda_array_interface__."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 2, "strides": None}


class Octree:
    """The Morton octree of src/LpmOctree.cpp built on the device (include/lpm_octree.h) over
    float64 (n, 3) device points; `arrays()` copies its device arrays into torch tensors.
    fixed_levels: the sync-free build (LPM_OCTREE_FIXED_LEVELS): level l at base_address[l] with
    room for min(8^l, 8 n) nodes, its first nnodes_per_level[l] nodes filled."""

    def __init__(self, x: torch.Tensor, max_depth: int, neighbors: bool = True, stream=None,
                 fixed_levels: bool = False):
        assert x.dtype == torch.float64 and x.is_cuda and x.dim() == 2 and x.shape[1] == 3
        h = ctypes.c_void_p()
        bits = (1 if neighbors else 0) | (2 if fixed_levels else 0)
        L.check(L.lib().lpm_octree_build(_vp(x), x.stride(0), x.stride(1), x.shape[0], max_depth, bits,
                                         ctypes.byref(h), _stream(stream)))
        self._h = h
        d, nn, n = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64()
        L.lib().lpm_octree_info(h, ctypes.byref(d), ctypes.byref(nn), ctypes.byref(n), None, None, None)
        self.max_depth, self.nnodes, self.npoints = d.value, nn.value, n.value
        npl = (ctypes.c_int32 * (self.max_depth + 1))()
        base = (ctypes.c_int32 * (self.max_depth + 1))()
        box = (ctypes.c_double * 6)()
        L.lib().lpm_octree_info(h, None, None, None, npl, base, box)
        self.nnodes_per_level = np.array(npl[:], dtype=np.int32)
        self.base_address = np.array(base[:], dtype=np.int32)
        self.box = np.array(box[:])
        self.neighbors = neighbors

    def arrays(self) -> dict:
        ptrs = [ctypes.c_void_p() for _ in range(8)]
        L.lib().lpm_octree_arrays(self._h, *[ctypes.byref(p) for p in ptrs])
        nn, n = self.nnodes, self.npoints
        spec = [("keys", (nn,), "<u4"), ("pt_inds", (nn, 2), "<i4"), ("parents", (nn,), "<i4"),
                ("kids", (nn, 8), "<i4"), ("neighbors", (nn, 27), "<i4"), ("sorted_pts", (n, 3), "<f8"),
                ("orig_ids", (n,), "<i4"), ("pt_in_leaf", (n,), "<i4")]
        out = {}
        for (name, shape, ts), p in zip(spec, ptrs):
            if p.value is None:
                out[name] = None
                continue
            if ts == "<u4":  # torch has no uint32 arithmetic everywhere: read as int32, reinterpret on the host
                t = torch.as_tensor(_DeviceView(p.value, shape, "<i4"), device="cuda").clone()
                out[name] = t.cpu().numpy().view(np.uint32)
            else:
                out[name] = torch.as_tensor(_DeviceView(p.value, shape, ts), device="cuda").clone()
        return out

    def close(self):
        if self._h:
            L.lib().lpm_octree_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mesh_face_verts(seed: int, level: int) -> np.ndarray:
    """Face-to-vertex connectivity (nfaces x 3 or 4) of build_mesh(seed, level)."""
    _, nf, _ = mesh_counts(seed, level)
    vpf = ctypes.c_int()
    L.check(L.lib().lpm_mesh_face_verts(seed, level, None, ctypes.byref(vpf)))
    fv = np.zeros((nf, vpf.value), dtype=np.int32)
    L.check(L.lib().lpm_mesh_face_verts(seed, level, _np_ptr(fv), ctypes.byref(vpf)))
    return fv


# ----------------------------------------------------------------------------------------
# snapshots and VTK output (include/lpm_bve_snapshot.h)
# ----------------------------------------------------------------------------------------
def _state_stream(state: "BVEState", stream) -> ctypes.c_void_p:
    """The stream of a snapshot call: the caller's, else the current one for device state, else
    none (a state of host tensors needs no device)."""
    if stream is None and not state.vx.is_cuda:
        return ctypes.c_void_p(None)
    return _stream(stream)


def snapshot_write(path: str, state: "BVEState", seed: int, level: int, t: float = 0.0, dt: float = 0.0,
                   omega: float = 2 * PI, stream=None):
    st = state.c_struct()
    L.check(L.lib().lpm_bve_snapshot_write(path.encode(), ctypes.byref(st), seed, level, t, dt, omega,
                                           _state_stream(state, stream)))


def snapshot_info(path: str) -> dict:
    sd, lv, nv, nf = ctypes.c_int(), ctypes.c_int(), L.c_i64(), L.c_i64()
    t, dt, om = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    L.check(L.lib().lpm_bve_snapshot_info(path.encode(), ctypes.byref(sd), ctypes.byref(lv), ctypes.byref(nv),
                                          ctypes.byref(nf), ctypes.byref(t), ctypes.byref(dt), ctypes.byref(om)))
    return dict(seed=sd.value, level=lv.value, nverts=nv.value, nfaces=nf.value, t=t.value, dt=dt.value,
                omega=om.value)


def snapshot_read(path: str, state: "BVEState", stream=None) -> float:
    """Restores positions, vorticity and velocity into `state`; returns the snapshot's time."""
    st = state.c_struct()
    t = ctypes.c_double()
    L.check(L.lib().lpm_bve_snapshot_read(path.encode(), ctypes.byref(st), ctypes.byref(t),
                                          _state_stream(state, stream)))
    return t.value


def vtk_write(path: str, state: "BVEState", seed: int, level: int, stream=None):
    st = state.c_struct()
    L.check(L.lib().lpm_bve_vtk_write(path.encode(), ctypes.byref(st), seed, level, _state_stream(state, stream)))


# ----------------------------------------------------------------------------------------
# context
# ----------------------------------------------------------------------------------------
@dataclass
class BVEState:
    """Device arrays of one solve (the arguments of BVERK4::advance_timestep).  Snapshot and VTK
    calls also take a state of host tensors."""
    vx: torch.Tensor
    vzeta: torch.Tensor
    vvel: torch.Tensor
    fx: torch.Tensor
    fzeta: torch.Tensor
    fvel: torch.Tensor
    farea: torch.Tensor
    fmask: Optional[torch.Tensor]

    def c_struct(self) -> L.State:
        for name in ("vx", "vvel", "fx", "fvel"):
            t = getattr(self, name)
            assert t.dtype == torch.float64 and t.dim() == 2 and t.shape[1] == 3, name
        return L.State(self.vx.shape[0], self.fx.shape[0],
                       self.vx.data_ptr(), self.vx.stride(0), self.vx.stride(1),
                       self.vzeta.data_ptr(),
                       self.vvel.data_ptr(), self.vvel.stride(0), self.vvel.stride(1),
                       self.fx.data_ptr(), self.fx.stride(0), self.fx.stride(1),
                       self.fzeta.data_ptr(),
                       self.fvel.data_ptr(), self.fvel.stride(0), self.fvel.stride(1),
                       self.farea.data_ptr(), _mask_ptr(self.fmask))


class Context:
    """Owns an lpm_bve_ctx (plans, stage workspace, captured graphs) on one GPU."""

    def __init__(self, device: Optional[int] = None, autotune: bool = False, verbose: bool = False):
        self._lib = L.lib()
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        h = ctypes.c_void_p()
        opts = L.Opts(device, int(autotune), int(verbose))
        L.check(self._lib.lpm_bve_ctx_create(ctypes.byref(h), ctypes.byref(opts)))
        self.handle = h

    def close(self):
        if self.handle:
            self._lib.lpm_bve_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def invalidate(self):
        L.check(self._lib.lpm_bve_plan_invalidate(self.handle), self.handle)

    def set_timing(self, enable: bool):
        """Bracket every pair-kernel launch with CUDA events (RK4 steps then launch directly)."""
        L.check(self._lib.lpm_bve_ctx_set_timing(self.handle, int(enable)), self.handle)

    @staticmethod
    def shapes():
        """FP32C pair-kernel launch shapes compiled into the library: (threads, K, source tile, min blocks)."""
        n = L.lib().lpm_bve_ctx_shapes(None, None, None, None, 0)
        t, k, s, b = [(ctypes.c_int * n)() for _ in range(4)]
        L.lib().lpm_bve_ctx_shapes(t, k, s, b, n)
        return [(t[i], k[i], s[i], b[i]) for i in range(n)]

    def set_shape(self, shape=None):
        """Fix the FP32C launch shape (threads, K, source tile, min blocks) for plans built
        afterwards (None = default)."""
        t, k, s, b = shape if shape else (0, 0, 0, 0)
        L.check(self._lib.lpm_bve_ctx_set_shape(self.handle, t, k, s, b), self.handle)

    def set_treecode(self, degree: int = 8, theta: float = 0.6, leaf_points: int = 512, min_pairs: float = 1e9):
        """Tree-code parameters for calls with flags & TREECODE (include/lpm_bve.h); solves with
        fewer than min_pairs target x source pairs keep the direct sum."""
        L.check(self._lib.lpm_bve_ctx_set_treecode(self.handle, degree, theta, leaf_points, min_pairs), self.handle)

    def set_symmetric(self, min_leaves: int = 65536):
        """Solves with at least min_leaves leaf sources compute each leaf-leaf pair once (FP32C
        collocated velocity and RK4 steps; plans built afterwards); 0 = every solve."""
        L.check(self._lib.lpm_bve_ctx_set_symmetric(self.handle, int(min_leaves)), self.handle)

    def tree_stats(self) -> dict:
        """Octree depth and nodes, far clusters and pairs of the last tree-code evaluation."""
        d, nodes, far = ctypes.c_int(), L.c_i64(), L.c_i64()
        pairs, dp, fp = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        ph = (ctypes.c_double * 3)()
        L.check(self._lib.lpm_bve_ctx_tree_stats(self.handle, ctypes.byref(d), ctypes.byref(nodes), ctypes.byref(far),
                                                 ctypes.byref(pairs), ctypes.byref(dp), ctypes.byref(fp), ph),
                self.handle)
        return dict(depth=d.value, nodes=nodes.value, far_clusters=far.value, pairs=pairs.value,
                    direct_pairs=dp.value, far_pairs=fp.value, build_ms=ph[0], upward_ms=ph[1], list_ms=ph[2])

    def timing(self, reset: bool = True):
        """(summed pair-kernel milliseconds, launches) since the last reset."""
        ms, n = ctypes.c_double(), L.c_i64()
        L.check(self._lib.lpm_bve_ctx_timing(self.handle, ctypes.byref(ms), ctypes.byref(n), int(reset)),
                self.handle)
        return ms.value, n.value

    def velocity(self, tgt: Optional[torch.Tensor], src_x: torch.Tensor, src_zeta: torch.Tensor,
                 src_area: torch.Tensor, src_mask: Optional[torch.Tensor], u: Optional[torch.Tensor] = None,
                 psi: Optional[torch.Tensor] = None, flags: int = 0, eps: float = 0.0, stream=None):
        """u (and psi) at `tgt` (or at the sources themselves with flags & COLLOCATED)."""
        colloc = bool(flags & L.COLLOCATED)
        n = src_x.shape[0] if colloc else tgt.shape[0]
        if u is None and not (flags & L.NO_VELOCITY):
            u = torch.empty((n, 3), dtype=torch.float64, device=src_x.device)
        if psi is None and (flags & L.PSI):
            psi = torch.empty(n, dtype=torch.float64, device=src_x.device)
        src = L.Sources(_points(src_x), _vp(src_zeta), _vp(src_area), _mask_ptr(src_mask))
        tp = None if colloc else ctypes.byref(_points(tgt))
        us = (u.stride(0), u.stride(1)) if u is not None else (3, 1)
        rc = self._lib.lpm_bve_velocity(self.handle, tp, ctypes.byref(src), _vp(u), us[0], us[1], _vp(psi),
                                        flags, eps, _stream(stream))
        L.check(rc, self.handle)
        return u, psi

    def rk4_step(self, state: BVEState, dt: float, omega: float, nsteps: int = 1, flags: int = 0,
                 eps: float = 0.0, stream=None):
        st = state.c_struct()
        rc = self._lib.lpm_bve_rk4_step(self.handle, ctypes.byref(st), dt, omega, nsteps, flags, eps,
                                        _stream(stream))
        L.check(rc, self.handle)

    def rk4_increments(self, stage: int, nverts: int, nfaces: int, stream=None):
        """Stage increments (x_k, zeta_k) of the last RK4 step, host arrays in particle order."""
        vx = np.zeros((nverts, 3)); vz = np.zeros(nverts); fx = np.zeros((nfaces, 3)); fz = np.zeros(nfaces)
        L.check(self._lib.lpm_bve_rk4_increments(self.handle, stage, _np_ptr(vx), _np_ptr(vz), _np_ptr(fx),
                                                 _np_ptr(fz), _stream(stream)), self.handle)
        return vx, vz, fx, fz

    def errnorms(self, appx: torch.Tensor, exact: torch.Tensor, wt: Optional[torch.Tensor] = None,
                 skip: Optional[torch.Tensor] = None, abs_linf: bool = False, stream=None):
        """Relative (l1, l2, linf) of appx against exact on the device (ErrNorms::compute,
        src/LpmErrorNorms.cpp:26-70): float64 (n, 3) vectors or (n,) scalars, optional float64
        weights and a byte mask of entries to leave out."""
        assert appx.dtype == torch.float64 and exact.dtype == torch.float64 and appx.shape == exact.shape
        ncomp = 3 if appx.dim() == 2 else 1
        if ncomp == 3:
            assert appx.shape[1] == 3
            a_sc, e_sc = appx.stride(1), exact.stride(1)
        else:
            a_sc = e_sc = 0
        if wt is not None:
            assert wt.dtype == torch.float64 and wt.is_contiguous() and wt.shape[0] == appx.shape[0]
        if skip is not None:
            assert skip.dtype in (torch.uint8, torch.bool) and skip.is_contiguous()
        out = (ctypes.c_double * 3)()
        L.check(self._lib.lpm_errnorms(self.handle, appx.data_ptr(), appx.stride(0), a_sc, exact.data_ptr(),
                                       exact.stride(0), e_sc, _vp(wt), _vp(skip), appx.shape[0], ncomp,
                                       L.NORMS_ABS_LINF if abs_linf else 0, out, _stream(stream)), self.handle)
        return tuple(out)

    def ensemble(self, states: Sequence[BVEState], flags: int = 0, eps: float = 0.0, stream=None) -> "Ensemble":
        return Ensemble(self, states, flags, eps, stream)


class Ensemble:
    """Many independent solves advanced together (include/lpm_bve_ensemble.h)."""

    def __init__(self, ctx: Context, states: Sequence[BVEState], flags: int, eps: float, stream=None):
        self.ctx = ctx
        self.states = list(states)
        arr = (L.State * len(self.states))(*[s.c_struct() for s in self.states])
        h = ctypes.c_void_p()
        L.check(ctx._lib.lpm_bve_ensemble_create(ctx.handle, arr, len(self.states), flags, eps, _stream(stream),
                                                 ctypes.byref(h)), ctx.handle)
        self.handle = h

    def step(self, dt, omega, nsteps: int = 1, stream=None):
        m = len(self.states)
        dts = np.broadcast_to(np.asarray(dt, dtype=np.float64), (m,)).copy()
        oms = np.broadcast_to(np.asarray(omega, dtype=np.float64), (m,)).copy()
        rc = self.ctx._lib.lpm_bve_ensemble_step(self.handle, dts.ctypes.data_as(L.c_dp),
                                                 oms.ctypes.data_as(L.c_dp), nsteps, _stream(stream))
        L.check(rc, self.ctx.handle)

    def info(self):
        ns, ni, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        pairs, nbytes = L.c_i64(), ctypes.c_size_t()
        L.check(self.ctx._lib.lpm_bve_ensemble_info(self.handle, ctypes.byref(ns), ctypes.byref(ni), ctypes.byref(g),
                                                    ctypes.byref(pairs), ctypes.byref(nbytes)))
        return dict(nsolves=ns.value, nitems=ni.value, grid=g.value, pairs_per_eval=pairs.value,
                    device_bytes=nbytes.value)

    def close(self):
        if self.handle:
            self.ctx._lib.lpm_bve_ensemble_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def server_estimate(seed: int, level: int, flags: int = L.FP32C, nsteps: int = 1, dt: float = 0.01) -> int:
    """Device bytes a server with these flags reserves for one request on this mesh (host-only)."""
    opts = L.ServerOpts(0, 0, 0, flags, 0.0, 0)
    req = L.Request(seed, level, 0, 0, 0.1, dt, 2 * PI, nsteps)
    n = ctypes.c_size_t()
    L.check(L.lib().lpm_bve_server_estimate(ctypes.byref(opts), ctypes.byref(req), ctypes.byref(n)))
    return n.value


class Server:
    """Continuous-batching solve server on one GPU (include/lpm_bve_server.h).

    ``submit`` queues a request (mesh seed/level, RH54 + seeded Gaussian vortices, dt, Omega,
    step count) and returns its id at once; the server admits requests while their device
    footprint fits the HBM budget and advances every running solve by one RK4 step per
    iteration.  ``result`` returns the final state as host arrays.
    """

    def __init__(self, device: Optional[int] = None, budget_bytes: int = 0, max_active: int = 0,
                 flags: int = L.FP32C, eps: float = 0.0, host_ic: bool = False):
        self._lib = L.lib()
        dev = torch.cuda.current_device() if device is None else device
        opts = L.ServerOpts(dev, budget_bytes, max_active, flags, eps, int(host_ic))
        h = ctypes.c_void_p()
        rc = self._lib.lpm_bve_server_create(ctypes.byref(opts), ctypes.byref(h))
        if rc != L.LPM_OK:
            raise L.LpmError(rc, "server creation failed (see stderr)")
        self.handle = h

    def _check(self, rc):
        if rc != L.LPM_OK:
            raise L.LpmError(rc, self._lib.lpm_bve_server_last_error(self.handle).decode())
        return rc

    def submit(self, seed: int, level: int, dt: float, nsteps: int, omega: float = 2 * PI, ic_seed: int = 0,
               n_gaussians: int = 3, gauss_width: float = 0.1) -> int:
        req = L.Request(seed, level, ic_seed, n_gaussians, gauss_width, dt, omega, nsteps)
        rid = L.c_i64()
        self._check(self._lib.lpm_bve_server_submit(self.handle, ctypes.byref(req), ctypes.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout: Optional[float] = None) -> bool:
        """True when the request is done; False on timeout; raises if it failed or was cancelled."""
        rc = self._lib.lpm_bve_server_wait(self.handle, rid, -1.0 if timeout is None else float(timeout))
        if rc == L.LPM_ERR_TIMEOUT:
            return False
        self._check(rc)
        return True

    def status(self, rid: int) -> int:
        st = ctypes.c_int()
        self._check(self._lib.lpm_bve_server_status(self.handle, rid, ctypes.byref(st)))
        return st.value

    def cancel(self, rid: int):
        self._check(self._lib.lpm_bve_server_cancel(self.handle, rid))

    def result(self, rid: int) -> dict:
        nv, nf = L.c_i64(), L.c_i64()
        self._check(self._lib.lpm_bve_server_result(self.handle, rid, ctypes.byref(nv), ctypes.byref(nf),
                                                    None, None, None, None, None, None))
        nv, nf = nv.value, nf.value
        out = dict(vx=np.zeros((nv, 3)), vzeta=np.zeros(nv), vvel=np.zeros((nv, 3)),
                   fx=np.zeros((nf, 3)), fzeta=np.zeros(nf), fvel=np.zeros((nf, 3)))
        p = [_np_ptr(out[k]) for k in ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")]
        self._check(self._lib.lpm_bve_server_result(self.handle, rid, None, None, *p))
        return out

    def release(self, rid: int):
        self._check(self._lib.lpm_bve_server_release(self.handle, rid))

    def snapshot(self, rid: int, path: str):
        """Final state of a finished request as a snapshot file (restore with snapshot_read)."""
        self._check(self._lib.lpm_bve_server_snapshot(self.handle, rid, path.encode()))

    def timing(self, rid: int) -> dict:
        t, w, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self._lib.lpm_bve_server_timing(self.handle, rid, ctypes.byref(t), ctypes.byref(w),
                                                    ctypes.byref(r)))
        return dict(total_s=t.value, wait_s=w.value, run_s=r.value)

    def latency(self, quantiles=(0.5, 0.99)) -> list:
        q = np.asarray(quantiles, dtype=np.float64)
        out = np.zeros_like(q)
        self._check(self._lib.lpm_bve_server_latency(self.handle, q.ctypes.data_as(L.c_dp), q.size,
                                                     out.ctypes.data_as(L.c_dp)))
        return out.tolist()

    def stats(self) -> dict:
        c = L.ServerCounters()
        self._check(self._lib.lpm_bve_server_stats(self.handle, ctypes.byref(c)))
        return {name: getattr(c, name) for name, _ in L.ServerCounters._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self._lib.lpm_bve_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------------------------------
# reference-shaped containers
# ----------------------------------------------------------------------------------------
def _dev_vec(host: np.ndarray, device, layout: str) -> torch.Tensor:
    """(n, 3) float64 device tensor; layout 'left' = SoA strides (1, n) like Kokkos CUDA views."""
    t = torch.from_numpy(np.ascontiguousarray(host, dtype=np.float64))
    if layout == "left":
        return t.t().contiguous().to(device).t()
    return t.to(device)


class BVESphere:
    """The BVE problem on a uniformly refined sphere mesh (BVESphere<Seed>, src/LpmBVESphere.hpp:18-80).

    Field names follow the reference: physVerts/physFaces coordinates, relVort*, absVort*,
    streamFn*, velocity*, faces area and mask, and the Lagrangian copies of the coordinates.
    """

    def __init__(self, seed: int, level: int, omega: float = 2 * PI, layout: str = "left", device="cuda",
                 mesh: Optional[dict] = None):
        m = mesh if mesh is not None else build_mesh(seed, level)
        self.seed, self.level, self.layout, self.device = seed, level, layout, torch.device(device)
        self.mesh = m
        self.Omega = omega
        self.t = 0.0
        self.physVerts = _dev_vec(m["vx"], self.device, layout)
        self.physFaces = _dev_vec(m["fx"], self.device, layout)
        self.lagVerts = self.physVerts.clone()
        self.lagFaces = self.physFaces.clone()
        self.faces_area = torch.from_numpy(m["farea"]).to(self.device)
        self.faces_mask = torch.from_numpy(m["fmask"]).to(self.device)
        nv, nf = m["nverts"], m["nfaces"]
        z = lambda n: torch.zeros(n, dtype=torch.float64, device=self.device)  # noqa: E731
        self.relVortVerts, self.absVortVerts, self.streamFnVerts = z(nv), z(nv), z(nv)
        self.relVortFaces, self.absVortFaces, self.streamFnFaces = z(nf), z(nf), z(nf)
        self.velocityVerts = _dev_vec(np.zeros((nv, 3)), self.device, layout)
        self.velocityFaces = _dev_vec(np.zeros((nf, 3)), self.device, layout)

    def nvertsHost(self):
        return self.mesh["nverts"]

    def nfacesHost(self):
        return self.mesh["nfaces"]

    def nleaves(self):
        return self.mesh["nleaves"]

    def avg_mesh_size_radians(self):
        return math.sqrt(4 * PI / self.nfacesHost())

    def init_vorticity(self, ic: Callable[[np.ndarray], np.ndarray], ctx: Context, flags: int = L.FP64,
                       eps: float = 0.0):
        """Host IC evaluation, then psi and u at vertices and faces (src/LpmBVESphere.cpp:127-169)."""
        vx, fx = self.mesh["vx"], self.mesh["fx"]
        zv = ic(vx); zf = ic(fx)
        self.relVortVerts.copy_(torch.from_numpy(zv))
        self.absVortVerts.copy_(torch.from_numpy(zv + 2 * self.Omega * vx[:, 2]))
        self.relVortFaces.copy_(torch.from_numpy(zf))
        self.absVortFaces.copy_(torch.from_numpy(zf + 2 * self.Omega * fx[:, 2]))
        self.solve(ctx, flags, eps, psi=True)

    def solve(self, ctx: Context, flags: int = L.FP64, eps: float = 0.0, psi: bool = True):
        """Velocity (and stream function) at all vertices and faces from the face vorticity."""
        prec = flags & L.FP32C
        f = prec | (L.PSI if psi else 0)
        ctx.velocity(self.physVerts, self.physFaces, self.relVortFaces, self.faces_area, self.faces_mask,
                     u=self.velocityVerts, psi=self.streamFnVerts if psi else None, flags=f | L.MESH_TARGETS,
                     eps=eps)
        ctx.velocity(None, self.physFaces, self.relVortFaces, self.faces_area, self.faces_mask,
                     u=self.velocityFaces, psi=self.streamFnFaces if psi else None, flags=f | L.COLLOCATED, eps=eps)

    def state(self) -> BVEState:
        return BVEState(self.physVerts, self.relVortVerts, self.velocityVerts, self.physFaces, self.relVortFaces,
                        self.velocityFaces, self.faces_area, self.faces_mask)


class BVERK4:
    """RK4 stepper with the reference's interface (src/LpmBVERK4.hpp:13-65)."""

    def __init__(self, dt: float, Omega: float, ctx: Optional[Context] = None, flags: int = L.FP64,
                 eps: float = 0.0):
        self.dt, self.Omega = dt, Omega
        self.nverts = self.nfaces = 0
        self.ctx = ctx or Context()
        self.flags, self.eps = flags, eps

    def init(self, nv: int, nf: int):
        self.nverts, self.nfaces = nv, nf

    def advance_timestep(self, vx, vzeta, vvel, fx, fzeta, fvel, fa, fm, nsteps: int = 1):
        if vx.shape[0] != self.nverts or fx.shape[0] != self.nfaces:
            raise ValueError("advance_timestep: array sizes differ from init(nv, nf)")
        self.ctx.rk4_step(BVEState(vx, vzeta, vvel, fx, fzeta, fvel, fa, fm), self.dt, self.Omega, nsteps,
                          self.flags, self.eps)
