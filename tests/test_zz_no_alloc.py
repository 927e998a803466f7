"""lpm_bve_velocity_noalloc, called through the C ABI, against lpm_bve_velocity.

The entry point serves callers that own all device memory and cannot let the library call
cudaMalloc (e.g. a host model with a fixed memory pool, or a time loop inside a captured
CUDA graph).  It keeps its scratch in one static device array shared by every call, so the
test runs two different problems back to back on the same scratch and checks each result
against the allocating entry point within the FP32C tolerance used throughout the tests
(relative L2 <= 1e-6), plus bitwise repeatability of a repeated call.

The file is named to be collected last; it passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import _lib as L

pytestmark = pytest.mark.gpu

FP32C_TOL = 1e-6
MAX_FACES = 1 << 19


def _fn():
    f = L.lib().lpm_bve_velocity_noalloc
    f.argtypes = [ctypes.POINTER(L.Points), ctypes.POINTER(L.Sources), ctypes.c_void_p, L.c_i64, L.c_i64,
                  ctypes.c_void_p, ctypes.c_uint, ctypes.c_double, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _dev(a, layout="left"):
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64))
    if t.dim() == 2 and layout == "left":
        return t.t().contiguous().cuda().t()
    return t.cuda()


def _pts(x):
    return L.Points(x.data_ptr(), x.shape[0], x.stride(0), x.stride(1))


def _problem(seed, level, rseed):
    from lpmkokkos_gb300 import bve
    m = bve.build_mesh(seed, level)
    zf = bve.rh54_gaussians(rseed, 3)(m["fx"])
    return dict(vx=_dev(m["vx"]), fx=_dev(m["fx"], "right"), z=_dev(zf), a=_dev(m["farea"]),
                mask=torch.from_numpy(m["fmask"]).cuda(), leaf=torch.from_numpy(m["fmask"] == 0).cuda())


def _noalloc(prob, colloc, psi=True, eps=0.0):
    n = prob["fx"].shape[0] if colloc else prob["vx"].shape[0]
    u = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    p = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    src = L.Sources(_pts(prob["fx"]), prob["z"].data_ptr(), prob["a"].data_ptr(), prob["mask"].data_ptr())
    tgt = None if colloc else ctypes.byref(_pts(prob["vx"]))
    flags = P.FP32C | (P.COLLOCATED if colloc else 0) | (P.PSI if psi else 0)
    rc = _fn()(tgt, ctypes.byref(src), u.data_ptr(), u.stride(0), u.stride(1), p.data_ptr() if psi else None,
               flags, eps, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.LPM_OK
    return u, p


def _reference(ctx, prob, colloc, eps=0.0):
    flags = P.FP32C | P.PSI | (P.COLLOCATED if colloc else 0)
    return ctx.velocity(None if colloc else prob["vx"], prob["fx"], prob["z"], prob["a"], prob["mask"],
                        flags=flags, eps=eps)


def _l2(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def test_noalloc_matches_allocating_entry_point_two_calls():
    torch.cuda.set_device(0)
    ctx = P.bve.Context(0)
    first = _problem(0, 5, 11)        # icosahedral level 5: vertex targets
    second = _problem(1, 5, 12)       # cubed sphere level 5: face targets, different mask and size
    u1, p1 = _noalloc(first, colloc=False)
    u2, p2 = _noalloc(second, colloc=True)
    torch.cuda.synchronize()
    r1u, r1p = _reference(ctx, first, colloc=False)
    r2u, r2p = _reference(ctx, second, colloc=True)
    torch.cuda.synchronize()
    leaf = second["leaf"]
    assert _l2(u1, r1u) <= FP32C_TOL and _l2(p1, r1p) <= FP32C_TOL
    assert _l2(u2[leaf], r2u[leaf]) <= FP32C_TOL and _l2(p2[leaf], r2p[leaf]) <= FP32C_TOL
    assert torch.isfinite(u1).all() and torch.isfinite(u2[leaf]).all()
    # the scratch now holds the second problem; repeating the first call reproduces it exactly
    u3, p3 = _noalloc(first, colloc=False)
    torch.cuda.synchronize()
    assert torch.equal(u3, u1) and torch.equal(p3, p1)
    ctx.close()


def test_noalloc_rejects_oversized_and_fp64():
    torch.cuda.set_device(0)
    prob = _problem(0, 2, 3)
    u = torch.empty((prob["vx"].shape[0], 3), dtype=torch.float64, device="cuda")
    big = L.Sources(L.Points(prob["fx"].data_ptr(), MAX_FACES + 1, 3, 1), prob["z"].data_ptr(),
                    prob["a"].data_ptr(), None)
    rc = _fn()(ctypes.byref(_pts(prob["vx"])), ctypes.byref(big), u.data_ptr(), u.stride(0), u.stride(1), None,
               P.FP32C, 0.0, None)
    assert rc == L.LPM_ERR_NOT_SUPPORTED
    src = L.Sources(_pts(prob["fx"]), prob["z"].data_ptr(), prob["a"].data_ptr(), prob["mask"].data_ptr())
    rc = _fn()(ctypes.byref(_pts(prob["vx"])), ctypes.byref(src), u.data_ptr(), u.stride(0), u.stride(1), None,
               P.FP64, 0.0, None)
    assert rc == L.LPM_ERR_NOT_SUPPORTED


def test_noalloc_nan_target_at_tile_middle():
    """A target with an inf/NaN position (a masked parent that coincides with a leaf) in the
    middle of a target tile leaves the other targets of the tile finite."""
    torch.cuda.set_device(0)
    prob = _problem(0, 4, 5)
    vx = prob["vx"].clone()
    ref, _ = _noalloc(prob, colloc=False, psi=False)
    vx[256] = float("nan")
    prob2 = dict(prob, vx=vx)
    got, _ = _noalloc(prob2, colloc=False, psi=False)
    torch.cuda.synchronize()
    keep = torch.ones(vx.shape[0], dtype=torch.bool, device="cuda"); keep[256] = False
    assert torch.isfinite(got[keep]).all()
    assert _l2(got[keep], ref[keep]) <= FP32C_TOL
