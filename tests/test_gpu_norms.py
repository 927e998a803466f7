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
