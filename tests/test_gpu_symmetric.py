"""The symmetric leaf x leaf kernel (pairFP32CSym): FP32C collocated velocity and RK4 steps of a
single solve compute each unordered leaf pair once.  Checked over vertices and leaf faces:
  against the oracle                             : relative L2 <= 1e-6 (the FP32C bar)
  against the plain kernel (LPM_BVE_NO_SYMMETRIC): relative L2 <= 1e-6 (same sums, other rounding)
  repeated evaluations                           : bitwise (fixed-point reverse sums are order-free)
on meshes whose leaf count is and is not a multiple of the 1,024-leaf tile, smaller than one
tile, with no mask (every face a source), with eps > 0, with masked-target skipping and without
the Newton step.  Masked parents are left out, as everywhere: each sits ~1e-6 from its middle
child, and that near-singular pair makes its value ill-conditioned (the two kernels' different
target tiles give parents that differ by ~1e-3; FP64 knows them only to ~4e-4)."""
import math

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu

TOL = 1e-6
OMEGA = 2 * math.pi


@pytest.fixture(scope="module")
def sctx(native):
    """A context that takes the symmetric kernel at every size (the default starts at 65,536
    leaf sources), so that small, ragged and single-tile meshes exercise it."""
    c = bve.Context(0)
    c.set_symmetric(0)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def _fresh(sctx):
    yield
    sctx.invalidate()


def _l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _setup(seed, level, rseed=7, mask=True):
    m = bve.build_mesh(seed, level)
    z = bve.rh54_gaussians(rseed, 3)(m["fx"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    fx = torch.from_numpy(m["fx"]).t().contiguous().cuda().t()
    mk = dev(m["fmask"]) if mask else None
    return m, fx, dev(z), dev(m["farea"]), mk, z


@pytest.mark.parametrize("seed,level", [(0, 0), (1, 2), (0, 3), (1, 4), (0, 5), (1, 5), (0, 6)])
def test_collocated_against_oracle_and_plain_kernel(sctx, oracle, seed, level):
    ctx = sctx
    m, fx, z, a, mk, zh = _setup(seed, level)
    leaf = m["fmask"] == 0
    u_sym, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED)
    u_pln, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED | P.NO_SYMMETRIC)
    torch.cuda.synchronize()
    _, ref = oracle.velocity(m["vx"][:0], m["fx"], zh, m["farea"], m["fmask"])
    us, up = u_sym.cpu().numpy()[leaf], u_pln.cpu().numpy()[leaf]
    assert _l2(us, ref[leaf]) <= TOL, _l2(us, ref[leaf])
    assert _l2(us, up) <= TOL, _l2(us, up)


def test_no_mask_every_face_a_source(sctx, oracle):
    """No mask pointer: all 6,820 faces of icosahedral level 4 are sources and symmetric-kernel
    leaves (not a multiple of the tile), parents included.  Parents have zero area, so the true
    leaves' values are the well-conditioned ones compared here; a leaf with a zero-area parent
    exactly on it is NaN in the reference (0/0) and left out."""
    m, fx, z, a, _, zh = _setup(0, 4, mask=False)
    u, _ = sctx.velocity(None, fx, z, a, None, flags=P.FP32C | P.COLLOCATED)
    torch.cuda.synchronize()
    nomask = np.zeros(m["nfaces"], np.uint8)
    _, ref = oracle.velocity(m["vx"][:0], m["fx"], zh, m["farea"], nomask)
    leaf = (m["fmask"] == 0) & np.isfinite(ref).all(axis=1)
    assert leaf.sum() > 0.95 * (m["fmask"] == 0).sum()
    assert _l2(u.cpu().numpy()[leaf], ref[leaf]) <= TOL


def test_repeatable_bitwise(sctx):
    ctx = sctx
    m, fx, z, a, mk, _ = _setup(0, 5)
    u1, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED)
    u1 = u1.clone()
    u2, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED)
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(u1), torch.nan_to_num(u2))


@pytest.mark.parametrize("extra", [0, P.SKIP_MASKED_TARGETS, P.RCP_APPROX])
def test_rk4_against_fp64_and_plain(sctx, extra):
    """Three RK4 steps at icosahedral level 5 with the symmetric kernel, against the FP64 RK4
    (FP32C bar) and against the plain FP32C kernel."""
    runs = {}
    for name, flags in (("sym", P.FP32C | extra), ("plain", P.FP32C | P.NO_SYMMETRIC | extra),
                        ("fp64", P.FP64 | (extra & P.SKIP_MASKED_TARGETS))):
        s = bve.BVESphere(0, 5)
        s.init_vorticity(bve.rh54_gaussians(11, 3), sctx, flags=P.FP64)
        sctx.rk4_step(s.state(), 0.005, OMEGA, 3, flags=flags)
        torch.cuda.synchronize()
        runs[name] = s
    leaf = runs["fp64"].mesh["fmask"] == 0
    for attr in ("velocityVerts", "velocityFaces", "relVortFaces", "physFaces"):
        g = getattr(runs["sym"], attr).cpu().numpy()
        r = getattr(runs["fp64"], attr).cpu().numpy()
        q = getattr(runs["plain"], attr).cpu().numpy()
        if attr != "velocityVerts":
            g, r, q = g[leaf], r[leaf], q[leaf]
        assert _l2(g, r) <= TOL, (attr, _l2(g, r))
        assert _l2(g, q) <= TOL, (attr, _l2(g, q))


def test_eps_and_stream_function(sctx, oracle):
    """eps = 0.01 with the stream function: the symmetric kernel forms log2(2q) - 1 once per
    unordered pair for both directions; velocity and stream function meet the bar against the
    oracle, and the plain kernel's stream function (LPM_BVE_NO_SYMMETRIC) agrees to the same bar."""
    ctx = sctx
    m, fx, z, a, mk, zh = _setup(1, 5)
    leaf = m["fmask"] == 0
    u, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED, eps=0.01)
    u = u.clone()
    u2, p2 = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED | P.PSI, eps=0.01)
    u2, p2 = u2.clone(), p2.clone()
    u3, p3 = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED | P.PSI | P.NO_SYMMETRIC, eps=0.01)
    torch.cuda.synchronize()
    _, ref, _, rp = oracle.velocity(m["vx"][:0], m["fx"], zh, m["farea"], m["fmask"], eps=0.01, psi=True)
    assert _l2(u.cpu().numpy()[leaf], ref[leaf]) <= TOL
    assert _l2(u2.cpu().numpy()[leaf], ref[leaf]) <= TOL
    # (not bit-equal to u: with PSI the diagonal tile takes the symmetric sweep, not the plain tile)
    assert _l2(p2.cpu().numpy()[leaf], rp[leaf]) <= TOL
    assert _l2(p3.cpu().numpy()[leaf], rp[leaf]) <= TOL
    assert not torch.equal(p2, p3)   # the symmetric kernel ran


@pytest.mark.parametrize("seed,level,eps", [(0, 4, 0.0), (1, 4, 0.0), (0, 5, 0.05)])
def test_stream_function_vertices_and_faces(sctx, oracle, seed, level, eps):
    """BVESphere.solve with the stream function: vertices (plain kernel over all sources) and
    leaf faces (symmetric kernel), eps 0 included (the logs of the smallest separations),
    against the oracle."""
    from lpmkokkos_gb300 import bve
    s = bve.BVESphere(seed, level, layout="left")
    s.init_vorticity(bve.rh54_gaussians(31 + level, 3), sctx, flags=P.FP64)
    s.solve(sctx, flags=P.FP32C, eps=eps, psi=True)
    torch.cuda.synchronize()
    m = s.mesh
    leaf = m["fmask"] == 0
    uv, uf, pv, pf = oracle.velocity(m["vx"], m["fx"], s.relVortFaces.cpu().numpy(), m["farea"], m["fmask"],
                                     eps=eps, psi=True)
    assert _l2(s.velocityVerts.cpu().numpy(), uv) <= TOL
    assert _l2(s.velocityFaces.cpu().numpy()[leaf], uf[leaf]) <= TOL
    assert _l2(s.streamFnVerts.cpu().numpy(), pv) <= TOL
    assert _l2(s.streamFnFaces.cpu().numpy()[leaf], pf[leaf]) <= TOL


def test_size_threshold(ctx):
    """The layout is a per-solve choice: below the threshold a solve's bits equal the plain
    kernel's (LPM_BVE_NO_SYMMETRIC), at or above it the symmetric kernel runs (other rounding,
    same bar).  The default threshold is 65,536 leaf sources."""
    ctx.set_symmetric(6000)
    try:
        for seed, level, sym in ((0, 4, False), (1, 5, True)):   # 5,120 and 6,144 leaves
            m, fx, z, a, mk, _ = _setup(seed, level)
            leaf = torch.from_numpy(m["fmask"] == 0).cuda()
            u, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED)
            u = u.clone()
            q, _ = ctx.velocity(None, fx, z, a, mk, flags=P.FP32C | P.COLLOCATED | P.NO_SYMMETRIC)
            torch.cuda.synchronize()
            same = torch.equal(u[leaf], q[leaf])
            assert same != sym, (seed, level)
            assert _l2(u[leaf].cpu().numpy(), q[leaf].cpu().numpy()) <= TOL
    finally:
        ctx.set_symmetric(65536)
