"""Flags of the C ABI that change what is computed (include/lpm_bve.h):

  * LPM_BVE_RENORM: RK4 positions renormalised to |x| = 1 after the combine, as the oracle's
    RK4 with renormalisation (max-rel 1e-12 in FP64), |x| = 1 to 1e-15;
  * LPM_BVE_SKIP_MASKED_TARGETS: masked (divided) faces are neither evaluated nor advanced --
    their output arrays keep their contents -- and every vertex and leaf equals the run
    without the flag bit for bit in FP64 (per-target sums do not depend on the other targets);
  * LPM_BVE_RCP_APPROX: FP32C without the Newton step stays within the FP32C bar (1e-6
    relative L2 against FP64) and differs from the Newton result.
"""
import math

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi


def _sphere(ctx, seed, level, prec, rseed=17):
    s = bve.BVESphere(seed, level)
    s.init_vorticity(bve.rh54_gaussians(rseed, 3), ctx, flags=prec)
    torch.cuda.synchronize()
    return s


def _host(s):
    return [t.cpu().numpy().copy() for t in (s.physVerts, s.relVortVerts, s.velocityVerts, s.physFaces,
                                             s.relVortFaces, s.velocityFaces)]


def test_renorm_matches_oracle(ctx, oracle):
    s = _sphere(ctx, 0, 3, P.FP64)
    h = _host(s)
    ctx.rk4_step(s.state(), 0.01, OMEGA, 3, flags=P.FP64 | P.RENORM)
    torch.cuda.synchronize()
    ref = oracle.rk4(*h, s.mesh["farea"], s.mesh["fmask"], 0.01, OMEGA, 3, renorm=True)
    got = _host(s)
    leaf = s.mesh["fmask"] == 0
    for k in range(6):
        g, r = got[k], ref[k]
        if k >= 3:
            g, r = g[leaf], r[leaf]
        assert np.abs(g - r).max() <= 1e-12 * np.abs(r).max(), k
    for x in (got[0], got[3][leaf]):
        assert np.abs(np.linalg.norm(x, axis=1) - 1).max() <= 1e-15


def test_skip_masked_targets(ctx):
    a = _sphere(ctx, 0, 3, P.FP64)
    b = _sphere(ctx, 0, 3, P.FP64)
    masked = torch.from_numpy(b.mesh["fmask"] != 0).cuda()
    leaf = ~masked
    before = b.physFaces[masked].clone()
    ctx.rk4_step(a.state(), 0.01, OMEGA, 2, flags=P.FP64)
    ctx.rk4_step(b.state(), 0.01, OMEGA, 2, flags=P.FP64 | P.SKIP_MASKED_TARGETS)
    torch.cuda.synchronize()
    assert torch.equal(a.physVerts, b.physVerts) and torch.equal(a.velocityVerts, b.velocityVerts)
    assert torch.equal(a.physFaces[leaf], b.physFaces[leaf]) and torch.equal(a.relVortFaces[leaf], b.relVortFaces[leaf])
    assert torch.equal(b.physFaces[masked], before)           # masked faces are not advanced
    # the velocity entry point: masked face outputs keep their contents
    u = torch.full((b.physFaces.shape[0], 3), 7.0, dtype=torch.float64, device="cuda")
    ctx.velocity(None, b.physFaces, b.relVortFaces, b.faces_area, b.faces_mask, u=u,
                 flags=P.FP64 | P.COLLOCATED | P.SKIP_MASKED_TARGETS)
    full, _ = ctx.velocity(None, b.physFaces, b.relVortFaces, b.faces_area, b.faces_mask,
                           flags=P.FP64 | P.COLLOCATED)
    torch.cuda.synchronize()
    assert (u[masked] == 7.0).all()
    assert torch.equal(u[leaf], full[leaf])


def test_rcp_approx_within_fp32c_bar(ctx):
    s = _sphere(ctx, 0, 5, P.FP64)
    src = (s.physFaces, s.relVortFaces, s.faces_area, s.faces_mask)
    u64, _ = ctx.velocity(s.physVerts, *src, flags=P.FP64)
    u32, _ = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS)
    ur, _ = ctx.velocity(s.physVerts, *src, flags=P.FP32C | P.MESH_TARGETS | P.RCP_APPROX)
    torch.cuda.synchronize()
    err = (torch.linalg.norm(ur - u64) / torch.linalg.norm(u64)).item()
    assert err <= 1e-6, err
    assert not torch.equal(ur, u32)
