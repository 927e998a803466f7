"""Committed golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the
oracle) checked on CPU (oracle regenerates them) and on GPU (FP64 and FP32C paths).

Masked parent faces are excluded from value comparisons (they coincide with leaves and
are inf/nan in the reference too); mesh arrays must match exactly.
"""
import math
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [(0, "bve_icos_L2.npz"), (1, "bve_cube_L2.npz")]
SEED, NG, DT, OMEGA, NSTEPS = 20261203, 2, 0.01, 2 * math.pi, 2


def _load(name):
    return dict(np.load(os.path.join(HERE, name)))


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("kind,name", CASES)
def test_oracle_reproduces_fixture(oracle, kind, name):
    g = _load(name)
    m = oracle.mesh(kind, 2)
    for k in ("vx", "fx", "farea", "fmask"):
        assert np.array_equal(m[k], g[k]), k
    zf = oracle.rh54_gaussians(m["fx"], SEED, NG)
    leaf = g["fmask"] == 0
    assert _rel(zf, g["fzeta"]) <= 1e-14
    uv, uf, pv, pf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"], psi=True)
    assert _rel(uv, g["vu"]) <= 1e-13 and _rel(uf[leaf], g["fu"][leaf]) <= 1e-13
    assert _rel(pv, g["vpsi"]) <= 1e-13 and _rel(pf[leaf], g["fpsi"][leaf]) <= 1e-13
    out = oracle.rk4(m["vx"], g["vzeta"], uv, m["fx"], zf, uf, m["farea"], m["fmask"], DT, OMEGA, NSTEPS)
    assert _rel(out[0], g["rk_vx"]) <= 1e-13
    assert _rel(out[4][leaf], g["rk_fzeta"][leaf]) <= 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", CASES)
def test_gpu_matches_fixture(ctx, kind, name):
    import torch

    import lpmkokkos_gb300 as P
    from lpmkokkos_gb300 import bve
    g = _load(name)
    leaf = g["fmask"] == 0
    for prec, tol in ((P.FP64, 1e-12), (P.FP32C, 1e-6)):
        s = bve.BVESphere(kind, 2)
        assert np.array_equal(s.mesh["fx"], g["fx"])
        s.relVortVerts.copy_(torch.from_numpy(g["vzeta"]))
        s.relVortFaces.copy_(torch.from_numpy(g["fzeta"]))
        s.solve(ctx, flags=prec, psi=True)
        torch.cuda.synchronize()
        fu = s.velocityFaces.cpu().numpy()[leaf]
        u = np.concatenate([s.velocityVerts.cpu().numpy(), fu])
        want = np.concatenate([g["vu"], g["fu"][leaf]])
        err = _rel(u, want) if prec == P.FP64 else np.linalg.norm(u - want) / np.linalg.norm(want)
        assert err <= tol, (prec, err)
        ctx.rk4_step(s.state(), DT, OMEGA, NSTEPS, flags=prec)
        torch.cuda.synchronize()
        x = np.concatenate([s.physVerts.cpu().numpy(), s.physFaces.cpu().numpy()[leaf]])
        wx = np.concatenate([g["rk_vx"], g["rk_fx"][leaf]])
        assert _rel(x, wx) <= tol, (prec, _rel(x, wx))
