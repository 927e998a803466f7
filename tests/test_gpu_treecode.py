"""Tree-code evaluation (LPM_BVE_TREECODE, include/lpm_bve.h) against the direct sums.

The tree code is an approximation outside the reference: far source clusters act through
chart-interpolated proxies (lpmkokkos_gb300/csrc/tree.hpp).  Its bar is the FP32C bar --
relative L2 <= 1e-6 against the FP64 direct sum -- at the default parameters (degree 8,
theta 0.6, 512 sources per leaf; measured 8e-8 at icosahedral levels 6-7 and 1.2e-7 at level 8).
Masked icosahedral parents lie within ~1e-6 of a leaf, so their velocities are dominated by that
near-singular pair in every path (some inf/NaN).  Comparisons therefore take vertices and leaf
faces."""
import math
import threading
import time

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu

TOL = 1e-6
OMEGA = 2 * math.pi


def _rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def _sphere(ctx, seed, level):
    s = bve.BVESphere(seed, level)
    s.init_vorticity(bve.rh54_gaussians(7, 3), ctx, flags=P.FP32C)
    torch.cuda.synchronize()
    leaf = torch.from_numpy(s.mesh["fmask"] == 0).cuda()
    return s, (s.physFaces, s.relVortFaces, s.faces_area, s.faces_mask), leaf


@pytest.fixture
def tctx(ctx):
    ctx.set_treecode(min_pairs=0)  # default parameters, the tree code at every size
    yield ctx
    ctx.set_treecode()


@pytest.mark.parametrize("seed,level", [(0, 5), (0, 6), (1, 6)])
def test_velocity_and_psi_against_fp64(tctx, seed, level):
    ctx = tctx
    s, src, leaf = _sphere(ctx, seed, level)
    rv, pv = ctx.velocity(s.physVerts, *src, flags=P.FP64 | P.PSI)
    rf, pf = ctx.velocity(None, *src, flags=P.FP64 | P.COLLOCATED | P.PSI)
    tv, qv = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS | P.TREECODE | P.PSI)
    tf, qf = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE | P.PSI)
    torch.cuda.synchronize()
    errs = [_rel(tv, rv), _rel(tf[leaf], rf[leaf]), _rel(qv, pv), _rel(qf[leaf], pf[leaf])]
    print("tree code vs FP64 (u verts, u leaves, psi verts, psi leaves):", errs)
    assert max(errs) <= TOL, errs
    st = ctx.tree_stats()
    assert st["far_clusters"] > 0 and st["far_pairs"] > 0


def test_list_overflow_falls_back_to_direct_then_grows(tctx):
    """The list buffer is sized by a solve's first evaluation.  Shuffling the leaf positions in
    place (the cached plan keeps its tiles, which become spatially random, so almost nothing is
    far field) makes the next evaluation's lists outgrow the buffer: that evaluation sums every
    source for every tile (the exact direct sum) and reports it, and the one after runs with a
    grown buffer.  Both meet the FP32C bar against the FP64 sum of the shuffled state."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, 0, 5)
    nf, nl = s.physFaces.shape[0], int(leaf.sum())
    ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    torch.cuda.synchronize()
    assert ctx.tree_stats()["far_pairs"] > 0
    # leaves among leaves only: a few masked parents sit exactly on a leaf, and as sources they
    # would make exactly coincident pairs
    g = torch.Generator().manual_seed(5)
    idx = torch.nonzero(leaf).flatten()
    perm = idx[torch.randperm(idx.numel(), generator=g).cuda()]
    s.physFaces[idx] = s.physFaces[perm].clone()
    t2, _ = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    t2 = t2.clone()
    torch.cuda.synchronize()
    st2 = ctx.tree_stats()
    assert st2["far_pairs"] == 0 and st2["pairs"] == nf * nl, st2  # the direct fallback
    t3, _ = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    t3 = t3.clone()
    torch.cuda.synchronize()
    st3 = ctx.tree_stats()
    assert st3["pairs"] <= nf * nl, st3
    ref, _ = ctx.velocity(None, *src, flags=P.FP64 | P.COLLOCATED)
    torch.cuda.synchronize()
    e2, e3 = _rel(t2[leaf], ref[leaf]), _rel(t3[leaf], ref[leaf])
    assert e2 <= TOL and e3 <= TOL, (e2, e3)


def test_reproducible_and_work_reduction(tctx):
    ctx = tctx
    s, src, leaf = _sphere(ctx, 0, 6)
    a, _ = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    b, _ = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    torch.cuda.synchronize()
    assert torch.equal(a[leaf], b[leaf])
    st = ctx.tree_stats()
    nt, ns = s.physFaces.shape[0], int(leaf.sum())
    assert st["pairs"] < 0.5 * nt * ns  # measured 0.23 of the direct pairs at level 6
    assert st["pairs"] == st["direct_pairs"] + st["far_pairs"]


def test_all_direct_limit(tctx):
    """With a tiny opening parameter no cluster is far: every target meets every source directly
    (the pair count is exactly targets x sources) and the result is the FP32C direct sum to
    within FP32C rounding."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, 1, 4)
    ctx.set_treecode(8, 0.01, 512, 0)
    t, _ = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE)
    r, _ = ctx.velocity(None, *src, flags=P.FP64 | P.COLLOCATED)
    torch.cuda.synchronize()
    st = ctx.tree_stats()
    assert st["far_pairs"] == 0
    assert st["pairs"] == s.physFaces.shape[0] * int(leaf.sum())
    assert _rel(t[leaf], r[leaf]) <= TOL


def test_arbitrary_distinct_targets(tctx):
    """Targets that are not mesh points (the hi/lo 'precise' form), 200 of them 1e-4 from a leaf
    source (a hundredth of the mesh spacing; much closer and 1 - x.y underflows the FP64 sum)."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, 0, 6)
    rng = np.random.default_rng(11)
    x = rng.normal(size=(30000, 3))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    f = s.physFaces[leaf].cpu().numpy()[:200] + 1e-4
    x = np.concatenate([x, f / np.linalg.norm(f, axis=1, keepdims=True)])
    xt = torch.from_numpy(x).cuda()
    r, _ = ctx.velocity(xt, *src, flags=P.FP64)
    t, _ = ctx.velocity(xt, *src, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    assert _rel(t, r) <= TOL


def test_rk4_steps(tctx):
    """Five RK4 steps with the tree code against five FP64 direct steps."""
    ctx = tctx
    a, _, leaf = _sphere(ctx, 0, 5)
    b, _, _ = _sphere(ctx, 0, 5)
    ctx.rk4_step(a.state(), 0.005, OMEGA, 5, flags=P.FP64)
    ctx.rk4_step(b.state(), 0.005, OMEGA, 5, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    errs = [_rel(b.physVerts, a.physVerts), _rel(b.velocityVerts, a.velocityVerts),
            _rel(b.relVortVerts, a.relVortVerts), _rel(b.velocityFaces[leaf], a.velocityFaces[leaf])]
    print("rk4 tree vs FP64 (x, u, zeta verts; u leaves):", errs)
    assert max(errs) <= TOL, errs


def test_work_stays_low_over_rk4_steps(tctx):
    """Masked icosahedral parents coincide with a leaf and run away once the steps start; they
    must not widen their tiles (the far field would vanish).  After four level-6 steps the last
    evaluation still needs under 40 % of the direct pairs (measured 0.23 before any step)."""
    ctx = tctx
    s, _, leaf = _sphere(ctx, 0, 6)
    ctx.rk4_step(s.state(), 0.0025, OMEGA, 4, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    st = ctx.tree_stats()
    frac = st["pairs"] / ((s.physVerts.shape[0] + s.physFaces.shape[0]) * int(leaf.sum()))
    assert frac < 0.4, frac


def test_level8_against_fp32c_direct(tctx):
    """Full size (icosahedral level 8: 655,362 vertices, 1,310,720 leaf sources): the tree code
    against the FP32C direct sum (itself 7e-8 from FP64 at this size)."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, 0, 8)
    r, _ = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS)
    t, _ = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS | P.TREECODE)
    torch.cuda.synchronize()
    assert _rel(t, r) <= TOL
    st = ctx.tree_stats()
    assert st["pairs"] < 0.05 * s.physVerts.shape[0] * int(leaf.sum())


def test_invalid(ctx):
    for args in ((1, 0.6, 512), (11, 0.6, 512), (8, 0.0, 512), (8, 1.0, 512), (8, 0.6, 0), (8, 0.6, 512, -1.0)):
        with pytest.raises(RuntimeError):
            ctx.set_treecode(*args)
    s, src, _ = _sphere(ctx, 0, 2)
    with pytest.raises(RuntimeError) as e:
        ctx.velocity(None, *src, flags=P.FP64 | P.COLLOCATED | P.TREECODE)
    assert "FP32C" in str(e.value)
    ctx.set_treecode()


def test_regularised_kernel(tctx):
    """eps > 0 (the regularised kernel 1 / (1 - x.y + eps^2); absent from the reference)."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, 0, 6)
    rf, pf = ctx.velocity(None, *src, flags=P.FP64 | P.COLLOCATED | P.PSI, eps=0.01)
    tf, qf = ctx.velocity(None, *src, flags=P.FP32C | P.COLLOCATED | P.TREECODE | P.PSI, eps=0.01)
    torch.cuda.synchronize()
    assert max(_rel(tf[leaf], rf[leaf]), _rel(qf[leaf], pf[leaf])) <= TOL


@pytest.mark.parametrize("extra", [P.SKIP_MASKED_TARGETS, P.RENORM, P.RK4_FIX_QUIRK])
def test_rk4_flags_with_tree(tctx, extra):
    """The RK4 options combine with the tree code as with the direct sum (3 steps, icos L5)."""
    ctx = tctx
    a, _, leaf = _sphere(ctx, 0, 5)
    b, _, _ = _sphere(ctx, 0, 5)
    ctx.rk4_step(a.state(), 0.005, OMEGA, 3, flags=P.FP64 | extra)
    ctx.rk4_step(b.state(), 0.005, OMEGA, 3, flags=P.FP32C | P.TREECODE | extra)
    torch.cuda.synchronize()
    errs = [_rel(b.physVerts, a.physVerts), _rel(b.velocityVerts, a.velocityVerts),
            _rel(b.physFaces[leaf], a.physFaces[leaf]), _rel(b.relVortFaces[leaf], a.relVortFaces[leaf])]
    assert max(errs) <= TOL, errs


def test_cubed_sphere_rk4_including_parents(tctx):
    """On the cubed sphere a masked parent sits on its children's shared corner (not on a leaf):
    its velocity is finite, and the tree code must get it right too."""
    ctx = tctx
    a, _, _ = _sphere(ctx, 1, 5)
    b, _, _ = _sphere(ctx, 1, 5)
    ctx.rk4_step(a.state(), 0.005, OMEGA, 3, flags=P.FP64)
    ctx.rk4_step(b.state(), 0.005, OMEGA, 3, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    assert torch.isfinite(a.velocityFaces).all()
    errs = [_rel(b.velocityFaces, a.velocityFaces), _rel(b.physFaces, a.physFaces), _rel(b.velocityVerts, a.velocityVerts)]
    assert max(errs) <= TOL, errs


def test_ensemble_with_the_tree_code(tctx):
    """An ensemble of uneven solves with the tree code: each solve bit-identical to its own
    single-solve tree-code run, and within the bar of its FP64 direct run."""
    ctx = tctx
    specs = [(0, 4), (1, 5), (0, 6)]
    ens = [_sphere(ctx, *sp) for sp in specs]
    alone = [_sphere(ctx, *sp) for sp in specs]
    ref = [_sphere(ctx, *sp) for sp in specs]
    e = ctx.ensemble([t[0].state() for t in ens], flags=P.FP32C | P.TREECODE)
    e.step([0.005] * 3, [OMEGA] * 3, 2)
    for (a, _, leaf), (r, _, _) in zip(alone, ref):
        ctx.rk4_step(a.state(), 0.005, OMEGA, 2, flags=P.FP32C | P.TREECODE)
        ctx.rk4_step(r.state(), 0.005, OMEGA, 2, flags=P.FP64)
    torch.cuda.synchronize()
    for (x, _, leaf), (a, _, _), (r, _, _) in zip(ens, alone, ref):
        assert torch.equal(x.physVerts, a.physVerts) and torch.equal(x.velocityFaces[leaf], a.velocityFaces[leaf])
        assert _rel(x.velocityVerts, r.velocityVerts) <= TOL and _rel(x.physFaces[leaf], r.physFaces[leaf]) <= TOL
    e.close()


def test_server_with_the_tree_code(ctx):
    """A server created with LPM_BVE_TREECODE: the two icosahedral level-6 requests (1.2e10 pairs
    per evaluation, above min_pairs) are set up by the tree threads and stepped together in one
    tree class (a captured tree-code step, their evaluations on side streams); the cubed-sphere
    level-7 request (2.3e10 pairs) runs in a second tree class beside it, the small ones in the
    batched direct classes.  Every result equals the same request's result alone, bit for bit,
    and a tree request is within the bar of an FP64 single solve."""
    big = [(0, 6, 901), (0, 6, 905), (1, 7, 906)]
    small = [(0, 3, 902), (1, 4, 903), (1, 3, 904)]

    counters = []

    def run(specs):
        with bve.Server(0, flags=P.FP32C | P.TREECODE, host_ic=True) as srv:
            ids = [srv.submit(sk, lv, 0.0025, 3, ic_seed=seed, n_gaussians=3, gauss_width=0.1)
                   for sk, lv, seed in specs]
            for i in ids:
                assert srv.wait(i, 300.0)
            counters.append(srv.stats())
            return [srv.result(i) for i in ids]

    mix = run([small[0], big[0], small[1], big[1], big[2], small[2]])
    # the tree requests' direct-sum-equivalent pairs are kept apart from the pairs computed
    equiv = sum((1 + 4 * 3) * (lambda c: (c[0] + c[1]) * c[2])(bve.mesh_counts(sk, lv)) for sk, lv, _ in big)
    assert counters[0]["tree_equiv_pairs"] == equiv
    direct = sum((1 + 4 * 3) * (lambda c: (c[0] + c[1]) * c[2])(bve.mesh_counts(sk, lv)) for sk, lv, _ in small)
    assert counters[0]["pairs"] == direct
    alone = run([big[0]]) + run([big[1]]) + run([big[2]]) + run(small)
    for got, want in zip([mix[1], mix[3], mix[4], mix[0], mix[2], mix[5]], alone):
        for k in ("vx", "vvel", "fx", "fvel", "vzeta", "fzeta"):
            assert np.array_equal(got[k], want[k], equal_nan=True), k
    s = bve.BVESphere(0, 6)
    s.init_vorticity(bve.rh54_gaussians(901, 3, 0.1), ctx, flags=P.FP64)
    ctx.rk4_step(s.state(), 0.0025, OMEGA, 3, flags=P.FP64)
    torch.cuda.synchronize()
    ref = s.velocityVerts.cpu().numpy()
    assert np.linalg.norm(mix[1]["vvel"] - ref) <= TOL * np.linalg.norm(ref)


def test_server_tree_request_without_steps_and_shutdown():
    """Tree-code server edge cases.  A tree request with no steps returns its initial state (the
    initial velocity from its tree-code evaluation), equal to the same request alone, beside one
    with a step.  A server destroyed while a tree request is being set up or stepped returns (its
    evaluator and plan are released) instead of hanging."""
    keys = ("vx", "vvel", "fx", "fvel", "vzeta", "fzeta")
    spec = dict(ic_seed=911, n_gaussians=3, gauss_width=0.1)
    with bve.Server(0, flags=P.FP32C | P.TREECODE, host_ic=True) as srv:
        a = srv.submit(0, 6, 0.0025, 0, **spec)
        b = srv.submit(0, 6, 0.0025, 1, ic_seed=912, n_gaussians=3, gauss_width=0.1)
        assert srv.wait(a, 300.0) and srv.wait(b, 300.0)
        ra, rb = srv.result(a), srv.result(b)
        st = srv.stats()
    nv, nf, nl = bve.mesh_counts(0, 6)
    assert st["tree_equiv_pairs"] == (1 + 1 + 4) * (nv + nf) * nl
    assert np.isfinite(rb["vvel"]).all() and not np.array_equal(ra["fx"], rb["fx"])
    with bve.Server(0, flags=P.FP32C | P.TREECODE, host_ic=True) as srv:
        a2 = srv.submit(0, 6, 0.0025, 0, **spec)
        assert srv.wait(a2, 300.0)
        alone = srv.result(a2)
    for k in keys:
        assert np.array_equal(ra[k], alone[k], equal_nan=True), k
    srv = bve.Server(0, flags=P.FP32C | P.TREECODE)
    srv.submit(0, 7, 0.00125, 50, ic_seed=913, n_gaussians=3, gauss_width=0.1)
    time.sleep(0.5)
    t = threading.Thread(target=srv.close, daemon=True)
    t.start()
    t.join(120.0)
    assert not t.is_alive(), "server destroy did not return"


@pytest.mark.parametrize("seed,level", [(0, 0), (0, 1), (1, 0), (1, 2)])
def test_tiny_meshes(tctx, seed, level):
    """Octree depth 1, clusters smaller than a proxy set: everything is summed directly."""
    ctx = tctx
    s, src, leaf = _sphere(ctx, seed, level)
    r, _ = ctx.velocity(s.physVerts, *src, flags=P.FP64)
    t, _ = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS | P.TREECODE)
    torch.cuda.synchronize()
    assert _rel(t, r) <= TOL
    assert ctx.tree_stats()["far_pairs"] == 0


def test_no_sources_and_ragged_targets(tctx):
    """Every face masked: no sources, zero velocity; 1,001 distinct targets (not a tile multiple)."""
    ctx = tctx
    s, _, _ = _sphere(ctx, 0, 3)
    all_masked = torch.ones_like(s.faces_mask)
    x = torch.nn.functional.normalize(torch.randn(1001, 3, dtype=torch.float64, device="cuda"), dim=1)
    t, _ = ctx.velocity(x, s.physFaces, s.relVortFaces, s.faces_area, all_masked, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    assert torch.equal(t, torch.zeros_like(t))
    r, _ = ctx.velocity(x, s.physFaces, s.relVortFaces, s.faces_area, s.faces_mask, flags=P.FP64)
    t, _ = ctx.velocity(x, s.physFaces, s.relVortFaces, s.faces_area, s.faces_mask, flags=P.FP32C | P.TREECODE)
    torch.cuda.synchronize()
    assert _rel(t, r) <= TOL


def test_size_threshold_and_hybrid_ensemble(ctx):
    """Below min_pairs a solve keeps the direct sum: a TREECODE call on icosahedral level 5
    (7.7e8 pairs < 1e9) equals the direct FP32C sum of a plan with the tree's launch shape, and in an
    ensemble the small solves share one direct launch while the large one takes the tree code --
    every solve bit-identical to its own single-solve TREECODE run."""
    ctx.set_treecode()  # min_pairs 1e9
    specs = [(0, 4), (1, 5), (0, 5), (0, 6)]
    ens = [_sphere(ctx, *sp) for sp in specs]
    alone = [_sphere(ctx, *sp) for sp in specs]
    e = ctx.ensemble([t[0].state() for t in ens], flags=P.FP32C | P.TREECODE)
    e.step([0.005] * 4, [OMEGA] * 4, 2)
    kinds = []
    for a, _, _ in alone:
        ctx.rk4_step(a.state(), 0.005, OMEGA, 2, flags=P.FP32C | P.TREECODE)
        torch.cuda.synchronize()
        kinds.append(ctx.tree_stats()["far_pairs"] > 0)
    torch.cuda.synchronize()
    assert kinds == [False, False, False, True], kinds
    for (x, _, leaf), (a, _, _) in zip(ens, alone):
        assert torch.equal(x.physVerts, a.physVerts) and torch.equal(x.velocityFaces[leaf], a.velocityFaces[leaf])
    e.close()
