"""Device error norms (lpm_errnorms) against the oracle's ErrNorms::compute
(src/LpmErrorNorms.cpp:26-70): vectors and scalars, weights, LayoutLeft strides, a skip
mask, the reference's signed scalar linf and the magnitude variant.  The device reduction
order differs from the serial oracle, so agreement is to 1e-13 relative; two device calls on
the same data agree bitwise (fixed reduction order)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _close(got, ref):
    for k, g in zip(("l1", "l2", "linf"), got):
        assert abs(g - ref[k]) <= TOL * abs(ref[k]), (k, g, ref[k])


def _left(a):
    return torch.from_numpy(np.ascontiguousarray(a)).t().contiguous().cuda().t()


def test_vector_norms_match_oracle(ctx, oracle):
    rng = np.random.default_rng(5)
    n = 200_003
    exact = rng.normal(size=(n, 3))
    appx = exact + 1e-3 * rng.normal(size=(n, 3))
    wt = rng.uniform(0.5, 2.0, size=n)
    ref = oracle.errnorms_vec(appx, exact, wt)
    a, x, w = torch.from_numpy(appx).cuda(), torch.from_numpy(exact).cuda(), torch.from_numpy(wt).cuda()
    got = ctx.errnorms(a, x, w)
    _close(got, ref)
    assert ctx.errnorms(a, x, w) == got  # bitwise repeatable
    _close(ctx.errnorms(_left(appx), _left(exact), w), ref)  # LayoutLeft strides


def test_scalar_norms_signed_linf_and_abs(ctx, oracle):
    rng = np.random.default_rng(6)
    n = 77_777
    exact = rng.normal(size=n)
    appx = exact + 1e-2 * rng.normal(size=n)
    wt = np.ones(n)
    ref = oracle.errnorms_scalar(appx, exact, wt)
    a, x = torch.from_numpy(appx).cuda(), torch.from_numpy(exact).cuda()
    _close(ctx.errnorms(a, x), ref)
    e = appx - exact
    got = ctx.errnorms(a, x, abs_linf=True)
    assert abs(got[2] - np.abs(e).max() / np.abs(exact).max()) <= TOL * got[2]


def test_skip_mask_and_mesh_weights(ctx, oracle):
    """RH54 velocity at the leaves of an icosahedral level-4 mesh against the exact field,
    face-area weights, masked parents skipped on the device / removed for the oracle."""
    m = oracle.mesh(0, 4)
    z = oracle.ic_rh54(m["fx"])
    _, uf = oracle.velocity(m["vx"], m["fx"], z, m["farea"], m["fmask"])
    ex = oracle.rh54_velocity(m["fx"])
    leaf = m["fmask"] == 0
    ref = oracle.errnorms_vec(uf[leaf], ex[leaf], m["farea"][leaf])
    got = ctx.errnorms(torch.from_numpy(uf).cuda(), torch.from_numpy(ex).cuda(),
                       torch.from_numpy(m["farea"]).cuda(), torch.from_numpy(m["fmask"]).cuda())
    _close(got, ref)
    assert got[1] < 0.05


def test_invalid_arguments(ctx):
    from lpmkokkos_gb300 import _lib as L
    x = torch.zeros(4, 3, dtype=torch.float64, device="cuda")
    out = (__import__("ctypes").c_double * 3)()
    rc = L.lib().lpm_errnorms(ctx.handle, x.data_ptr(), 3, 1, x.data_ptr(), 3, 1, None, None, 4, 2, 0, out, None)
    assert rc == L.LPM_ERR_INVALID_ARGUMENT
    rc = L.lib().lpm_errnorms(ctx.handle, x.data_ptr(), 3, 1, x.data_ptr(), 3, 1, None, None, 0, 3, 0, out, None)
    assert rc == L.LPM_ERR_INVALID_ARGUMENT


def test_tangency_matches_oracle_bitwise(ctx, oracle):
    """lpm_sphere_tangency against the oracle's SphereVelocityTangentTestFunctor
    (src/LpmSphereTestKernels.hpp:11-25) on the velocity the device computed, as
    tests/LpmBVETest.cpp:160-163 runs it after a step: bit for bit (same order, no contraction),
    row-major and LayoutLeft, and |u . x| at rounding level for the tangent Biot-Savart field."""
    import math
    from lpmkokkos_gb300 import FP64, bve
    s = bve.BVESphere(1, 4)
    s.init_vorticity(bve.rh54_gaussians(11, 3), ctx, flags=FP64)
    ctx.rk4_step(s.state(), 0.01, 2 * math.pi, 1, flags=FP64)
    torch.cuda.synchronize()
    for x, u in ((s.physVerts, s.velocityVerts), (s.physFaces, s.velocityFaces)):
        ref = oracle.tangency(x.cpu().numpy(), u.cpu().numpy())
        got = bve.sphere_tangency(x, u)
        torch.cuda.synchronize()
        assert np.array_equal(got.cpu().numpy(), ref)
        xl = x.t().contiguous().t()
        ul = u.t().contiguous().t()
        assert np.array_equal(bve.sphere_tangency(xl, ul).cpu().numpy(), ref)
        assert np.abs(ref).max() <= 1e-14 * np.abs(u.cpu().numpy()).max()


def test_tangency_solid_body(ctx, oracle):
    """The solid-body field of tests/LpmBVETest.cpp:55-64: u = Omega (-y, x, 0) is tangent;
    u . x equals the oracle's bit for bit and is at most a few ulps of |u| (4.4e-16 here)."""
    from lpmkokkos_gb300 import bve
    m = bve.build_mesh(0, 3)
    x = m["vx"]
    u = 2 * np.pi * np.stack([-x[:, 1], x[:, 0], np.zeros(len(x))], axis=1)
    got = bve.sphere_tangency(torch.from_numpy(x).cuda(), torch.from_numpy(u).cuda())
    ref = oracle.tangency(x, u)
    assert np.array_equal(got.cpu().numpy(), ref)
    assert np.abs(ref).max() <= 1e-15


def test_tangency_invalid_arguments():
    from lpmkokkos_gb300 import _lib as L
    x = torch.zeros(4, 3, dtype=torch.float64, device="cuda")
    assert L.lib().lpm_sphere_tangency(x.data_ptr(), 3, 1, x.data_ptr(), 3, 1, -1, x.data_ptr(), None) \
        == L.LPM_ERR_INVALID_ARGUMENT
    assert L.lib().lpm_sphere_tangency(None, 3, 1, x.data_ptr(), 3, 1, 4, x.data_ptr(), None) \
        == L.LPM_ERR_INVALID_ARGUMENT
    assert L.lib().lpm_sphere_tangency(x.data_ptr(), 3, 1, x.data_ptr(), 3, 1, 0, None, None) == L.LPM_OK
