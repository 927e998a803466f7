"""Ensemble members and server requests checked directly against the oracle's RK4
(src/LpmBVERK4_Impl.hpp:42-130, restated in oracle/lpm_oracle.cpp), not only against the
single-solve CUDA path.  FP64; vertices and leaf faces; max |e| / max |ref| <= 1e-12.

  * a cubed-sphere level-3 member and an icosahedral level-4 member of a mixed FP64 ensemble
    (icosahedral levels 2-4 around them), 3 steps;
  * an FP64 server request (icosahedral level 3, RH54 + 3 seeded Gaussian vortices evaluated on
    the host, 3 steps) in a mix with other requests.
"""
import math

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi
TOL = 1e-12
KEYS = ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")


def _maxrel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check(got, ref, fmask, what):
    leaf = fmask == 0
    for k, name in enumerate(KEYS):
        g, r = got[k], ref[k]
        if k >= 3:
            g, r = g[leaf], r[leaf]
        err = _maxrel(g, r)
        assert err <= TOL, (what, name, err)


def _oracle_run(oracle, m, ic_seed, ng, dt, nsteps):
    zf = oracle.rh54_gaussians(m["fx"], ic_seed, ng)
    zv = oracle.rh54_gaussians(m["vx"], ic_seed, ng)
    uv, uf = oracle.velocity(m["vx"], m["fx"], zf, m["farea"], m["fmask"])
    return oracle.rk4(m["vx"], zv, uv, m["fx"], zf, uf, m["farea"], m["fmask"], dt, OMEGA, nsteps)


def test_mixed_ensemble_members_match_oracle(ctx, oracle):
    specs = [(0, 2, 11), (1, 3, 12), (0, 3, 13), (0, 4, 14), (0, 2, 15)]
    dts = [0.01, 0.008, 0.006, 0.005, 0.012]
    spheres = []
    for sd, lv, r in specs:
        s = bve.BVESphere(sd, lv)
        s.init_vorticity(bve.rh54_gaussians(r, 3), ctx, flags=P.FP64)
        spheres.append(s)
    ens = ctx.ensemble([s.state() for s in spheres], flags=P.FP64)
    ens.step(dts, [OMEGA] * len(specs), 3)
    torch.cuda.synchronize()
    ens.close()
    for i in (1, 3):   # the cubed-sphere level-3 and the icosahedral level-4 member
        sd, lv, r = specs[i]
        s = spheres[i]
        got = [t.cpu().numpy() for t in (s.physVerts, s.relVortVerts, s.velocityVerts, s.physFaces,
                                         s.relVortFaces, s.velocityFaces)]
        ref = _oracle_run(oracle, s.mesh, r, 3, dts[i], 3)
        _check(got, ref, s.mesh["fmask"], f"ensemble member seed {sd} level {lv}")


def test_fp64_server_request_in_a_mix_matches_oracle(oracle):
    torch.cuda.set_device(0)
    seed, level, dt, nsteps, ic_seed, ng = 0, 3, 0.01, 3, 21, 3
    with bve.Server(0, flags=P.FP64, host_ic=True) as srv:
        others = [srv.submit(1, 3, 0.01, 4, ic_seed=30 + k) for k in range(2)]
        rid = srv.submit(seed, level, dt, nsteps, ic_seed=ic_seed, n_gaussians=ng, gauss_width=0.1)
        others.append(srv.submit(0, 4, 0.005, 2, ic_seed=40))
        for r in (rid, *others):
            assert srv.wait(r, 600.0)
        got = srv.result(rid)
    m = bve.build_mesh(seed, level)
    ref = _oracle_run(oracle, m, ic_seed, ng, dt, nsteps)
    _check([got[k] for k in KEYS], ref, m["fmask"], "server request icos L3")
