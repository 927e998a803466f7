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


def _noalloc(prob, colloc, psi=True, eps=0.0, extra=0):
    n = prob["fx"].shape[0] if colloc else prob["vx"].shape[0]
    u = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    p = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    src = L.Sources(_pts(prob["fx"]), prob["z"].data_ptr(), prob["a"].data_ptr(), prob["mask"].data_ptr())
    tgt = None if colloc else ctypes.byref(_pts(prob["vx"]))
    flags = P.FP32C | (P.COLLOCATED if colloc else 0) | (P.PSI if psi else 0) | extra
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


TILE = 128 * 8   # targets per CTA of the no-allocation pair kernel


def test_noalloc_nan_target_at_tile_middle():
    """A target with an inf/NaN position (a masked parent that coincides with a leaf) at the
    middle of a target tile -- the slot the kernel takes as the tile centre -- leaves the other
    targets of the tile finite: the kernel falls back to the first sane target as the centre.
    A tile whose every target is NaN falls back to the origin and leaves other tiles unchanged."""
    torch.cuda.set_device(0)
    prob = _problem(0, 4, 5)                       # 2,562 vertices: tiles of 1024, 1024, 514
    n = prob["vx"].shape[0]
    for flags in (0, P.MESH_TARGETS):
        ref, _ = _noalloc(prob, colloc=False, psi=False, extra=flags)
        bad = torch.zeros(n, dtype=torch.bool, device="cuda")
        bad[min(TILE, n) // 2] = True               # centre slot of tile 0
        bad[TILE:2 * TILE] = True                   # every target of tile 1
        vx = prob["vx"].clone()
        vx[bad] = float("nan")
        got, _ = _noalloc(dict(prob, vx=vx), colloc=False, psi=False, extra=flags)
        torch.cuda.synchronize()
        keep = ~bad
        assert torch.isfinite(got[keep]).all()
        assert _l2(got[keep], ref[keep]) <= FP32C_TOL


def test_noalloc_refuses_flags_it_does_not_implement():
    """Flags of lpm_bve_velocity that this entry point does not implement return
    LPM_ERR_NOT_SUPPORTED instead of being ignored."""
    torch.cuda.set_device(0)
    prob = _problem(0, 2, 3)
    u = torch.empty((prob["vx"].shape[0], 3), dtype=torch.float64, device="cuda")
    src = L.Sources(_pts(prob["fx"]), prob["z"].data_ptr(), prob["a"].data_ptr(), prob["mask"].data_ptr())
    for bad in (P.TREECODE, P.RCP_APPROX, P.SKIP_MASKED_TARGETS):
        rc = _fn()(ctypes.byref(_pts(prob["vx"])), ctypes.byref(src), u.data_ptr(), u.stride(0), u.stride(1), None,
                   P.FP32C | bad, 0.0, None)
        assert rc == L.LPM_ERR_NOT_SUPPORTED, bad


def test_noalloc_at_its_face_ceiling_icos_level7():
    """Icosahedral level 7 (436,900 faces, under the 524,288-face limit), targets in the mesh's
    own order: vertices (with and without LPM_BVE_MESH_TARGETS) and every face (collocated),
    against lpm_bve_velocity."""
    torch.cuda.set_device(0)
    ctx = P.bve.Context(0)
    prob = _problem(0, 7, 17)
    leaf = prob["leaf"]
    for flags in (0, P.MESH_TARGETS):
        u, p = _noalloc(prob, colloc=False, extra=flags)
        ru, rp = ctx.velocity(prob["vx"], prob["fx"], prob["z"], prob["a"], prob["mask"],
                              flags=P.FP32C | P.PSI | P.MESH_TARGETS)
        torch.cuda.synchronize()
        assert _l2(u, ru) <= FP32C_TOL and _l2(p, rp) <= FP32C_TOL, (flags, _l2(u, ru), _l2(p, rp))
    u, p = _noalloc(prob, colloc=True)
    ru, rp = _reference(ctx, prob, colloc=True)
    torch.cuda.synchronize()
    assert _l2(u[leaf], ru[leaf]) <= FP32C_TOL and _l2(p[leaf], rp[leaf]) <= FP32C_TOL, \
        (_l2(u[leaf], ru[leaf]), _l2(p[leaf], rp[leaf]))
    ctx.close()


def test_noalloc_random_targets():
    """1,031 random unit vectors (no tile size divides the count; targets arbitrarily close to a
    source) get the hi/lo formulation and match lpm_bve_velocity's precise path."""
    torch.cuda.set_device(0)
    ctx = P.bve.Context(0)
    prob = _problem(0, 5, 19)
    rng = np.random.default_rng(1031)
    t = rng.normal(size=(1031, 3)); t /= np.linalg.norm(t, axis=1, keepdims=True)
    prob = dict(prob, vx=_dev(t))
    u, p = _noalloc(prob, colloc=False)
    ru, rp = ctx.velocity(prob["vx"], prob["fx"], prob["z"], prob["a"], prob["mask"], flags=P.FP32C | P.PSI)
    torch.cuda.synchronize()
    assert _l2(u, ru) <= FP32C_TOL and _l2(p, rp) <= FP32C_TOL, (_l2(u, ru), _l2(p, rp))
    ctx.close()
