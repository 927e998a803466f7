"""GPU parity against the CPU oracle at the benchmark configurations, on sampled targets.

Icosahedral level 7 (163,842 vertices, 436,900 faces, 327,680 leaf sources; RH54 + 3 Gaussian
vortices, eps 0) and level 8 (655,362 vertices, 1,747,620 faces, 1,310,720 leaf sources; RH54 + 8
Gaussian vortices, eps 0.01, stream function at every target) are the single-solve benchmark
workloads.  The oracle sums 4,096 random vertices and 4,096 random leaf faces over ALL sources
(each target of the reference's reductions is independent of the others,
src/LpmBVEKernels.hpp:140-186 and :263-305), on the initial state and again after two FP32C RK4
steps (src/LpmBVERK4_Impl.hpp:42-130).  Tolerances, as in the smaller parity tests:
  FP64  (pairFP64)  : max |e| / max |ref| <= 1e-12 for velocity and stream function
  FP32C (pairFP32C) : relative L2 <= 1e-6 for velocity and stream function
Face targets are the collocated (i != j) sums.  FP32C is evaluated at every target, as the
benchmark does, and sampled; the FP64 path is evaluated at the sampled targets only (a full
FP64 evaluation at level 8 takes minutes), its face sums split into two calls over a partition
of the sources (oracle/sampled_parity.py).  At level 7 the full FP64 collocated face launch is
also compared, velocity only.  The RK4 steps use FP32C, the benchmark's precision; the FP64
trajectory at these sizes (~15 min per level-8 step) is covered at small sizes elsewhere.
"""
import math

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from oracle import sampled_parity as SP

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32C_TOL = 1e-6

# (level, Gaussian vortices, initial-condition seed, eps): the level-7 and level-8 benchmark workloads
CONFIGS = {7: (3, 20261204, 0.0), 8: (8, 20261208, 0.01)}


def _fp32c_at(ctx, s, vidx, fidx, eps):
    s.solve(ctx, flags=P.FP32C, eps=eps, psi=True)
    torch.cuda.synchronize()
    return (s.velocityVerts.cpu().numpy()[vidx], s.streamFnVerts.cpu().numpy()[vidx],
            s.velocityFaces.cpu().numpy()[fidx], s.streamFnFaces.cpu().numpy()[fidx])


def _host(s):
    return (s.physVerts.cpu().numpy(), s.physFaces.cpu().numpy(), s.relVortFaces.cpu().numpy(),
            s.mesh["farea"], s.mesh["fmask"])


@pytest.mark.parametrize("level", [7, 8])
def test_bench_config_sampled_targets_match_oracle(ctx, oracle, level):
    from lpmkokkos_gb300 import bve
    ng, ic_seed, eps = CONFIGS[level]
    s = bve.BVESphere(0, level, layout="left")
    s.init_vorticity(bve.rh54_gaussians(ic_seed, ng), ctx, flags=P.FP32C, eps=eps)
    vidx, fidx = SP.sample_targets(s.mesh["nverts"], s.mesh["fmask"], seed=level)
    dt = 0.01 * 2.0 ** (4 - level)
    report = {}
    for when in ("initial", "after 2 RK4 steps"):
        if when != "initial":
            ctx.rk4_step(s.state(), dt, 2 * math.pi, 2, flags=P.FP32C, eps=eps)
            torch.cuda.synchronize()
        vx, fx, z, a, m = _host(s)
        ref = SP.oracle_at(vx, fx, z, a, m, vidx, fidx, eps=eps)
        # the velocity the RK4 step left in the state (its closing evaluation), FP32C
        if when != "initial":
            got_rk = (s.velocityVerts.cpu().numpy()[vidx], ref[1], s.velocityFaces.cpu().numpy()[fidx], ref[3])
            e = SP.compare(got_rk, ref)
            assert e["u_l2"] <= FP32C_TOL, (level, when, "rk4 state velocity", e)
        e32 = SP.compare(_fp32c_at(ctx, s, vidx, fidx, eps), ref)
        e64 = SP.compare(SP.gpu_fp64_at(ctx, P, torch, s.physVerts, s.physFaces, s.relVortFaces, s.faces_area,
                                        s.faces_mask, vidx, fidx, eps=eps), ref)
        report[when] = (e32, e64)
        assert e32["u_l2"] <= FP32C_TOL and e32["psi_l2"] <= FP32C_TOL, (level, when, e32)
        assert e32["u_faces_l2"] <= FP32C_TOL and e32["u_verts_l2"] <= FP32C_TOL, (level, when, e32)
        assert e64["u_maxrel"] <= FP64_TOL and e64["psi_maxrel"] <= FP64_TOL, (level, when, e64)
    print(f"level {level}: " + "; ".join(f"{k}: FP32C u {v[0]['u_l2']:.2e} psi {v[0]['psi_l2']:.2e}, "
                                         f"FP64 u {v[1]['u_maxrel']:.2e} psi {v[1]['psi_maxrel']:.2e}"
                                         for k, v in report.items()))


def test_level7_full_fp64_collocated_launch_matches_oracle(ctx, oracle):
    """The FP64 collocated launch over all 436,900 level-7 faces (the real face path of the
    RK4 step, not the sampled split), compared at the sampled leaf faces."""
    from lpmkokkos_gb300 import bve
    ng, ic_seed, eps = CONFIGS[7]
    s = bve.BVESphere(0, 7, layout="left")
    s.init_vorticity(bve.rh54_gaussians(ic_seed, ng), ctx, flags=P.FP32C, eps=eps)
    vidx, fidx = SP.sample_targets(s.mesh["nverts"], s.mesh["fmask"], seed=77)
    uf, _ = ctx.velocity(None, s.physFaces, s.relVortFaces, s.faces_area, s.faces_mask,
                         flags=P.FP64 | P.COLLOCATED, eps=eps)
    torch.cuda.synchronize()
    vx, fx, z, a, m = _host(s)
    ref = oracle.velocity_faces(fidx, fx, z, a, m, eps=eps)
    got = uf.cpu().numpy()[fidx]
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= FP64_TOL, err
