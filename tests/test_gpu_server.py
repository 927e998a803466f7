"""Continuous-batching server (include/lpm_bve_server.h) through the C ABI.

  * a request's final state is bitwise the same run alone and run in a mix of requests of
    other sizes that arrive while it runs (per-solve summation order is fixed);
  * in FP64 the server's result is bitwise the single-solve path's: BVESphere initial
    condition + velocity, then lpm_bve_rk4_step (itself pinned to the oracle at 1e-12);
  * a request with zero steps returns the initial state with its velocity;
  * the initial vorticity evaluated on the GPU (default) agrees with the host functions to
    1e-13 relative, and the steps from it to 1e-10 (FP64);
  * the HBM budget admits one request at a time when only one fits, rejects a request that
    can never fit, and a queued request can be cancelled;
  * invalid requests are rejected; stats and latency quantiles are consistent.
"""
import math
import time

import numpy as np
import pytest
import torch

import lpmkokkos_gb300 as P
from lpmkokkos_gb300 import _lib as L
from lpmkokkos_gb300 import bve

pytestmark = pytest.mark.gpu

OMEGA = 2 * math.pi
KEYS = ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")
WAIT = 600.0


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


def _alone(flags, spec):
    with bve.Server(0, flags=flags) as srv:
        rid = srv.submit(**spec)
        assert srv.wait(rid, WAIT)
        return srv.result(rid)


@pytest.mark.parametrize("flags", [P.FP32C, P.FP64])
def test_same_result_alone_and_in_the_mix(flags):
    torch.cuda.set_device(0)
    a_spec = dict(seed=0, level=4, dt=0.005, nsteps=5, ic_seed=7)
    b_spec = dict(seed=1, level=5, dt=0.0025, nsteps=3, ic_seed=8)
    alone_a, alone_b = _alone(flags, a_spec), _alone(flags, b_spec)
    long_level = 6 if flags == P.FP32C else 5  # FP64 pairs run at 1/64 of the FP32 rate
    with bve.Server(0, flags=flags) as srv:
        long_run = srv.submit(seed=0, level=long_level, dt=0.0025, nsteps=12, ic_seed=1)
        small = [srv.submit(seed=1, level=3, dt=0.01, nsteps=2 + s, ic_seed=s) for s in range(4)]
        time.sleep(0.05)
        a = srv.submit(**a_spec)
        time.sleep(0.02)
        b = srv.submit(**b_spec)
        late = [srv.submit(seed=0, level=5, dt=0.005, nsteps=2, ic_seed=10 + s) for s in range(3)]
        for rid in (long_run, a, b, *small, *late):
            assert srv.wait(rid, WAIT)
        st = srv.stats()
        got_a, got_b = srv.result(a), srv.result(b)
        # size classes: the small requests step several times per step of the long one
        small_done = max(srv.timing(r)["total_s"] for r in small)
        long_done = srv.timing(long_run)["total_s"]
    assert st["completed"] == 10 and st["failed"] == 0
    assert small_done < long_done, (small_done, long_done)
    assert st["max_running_seen"] >= 3, st  # the requests really shared launches
    for k in KEYS:
        assert _same(got_a[k], alone_a[k]), k
        assert _same(got_b[k], alone_b[k]), k
    leaf = bve.build_mesh(0, 4)["fmask"] == 0
    assert np.isfinite(got_a["fx"][leaf]).all() and np.isfinite(got_a["vvel"]).all()


def test_fp64_server_matches_single_solve_path(ctx):
    torch.cuda.set_device(0)
    seed, level, dt, nsteps, ic_seed, ng, width = 0, 3, 0.01, 3, 5, 3, 0.1
    with bve.Server(0, flags=P.FP64, host_ic=True) as srv:
        r0 = srv.submit(seed, level, dt, 0, ic_seed=ic_seed, n_gaussians=ng, gauss_width=width)
        r3 = srv.submit(seed, level, dt, nsteps, ic_seed=ic_seed, n_gaussians=ng, gauss_width=width)
        assert srv.wait(r0, WAIT) and srv.wait(r3, WAIT)
        init, got = srv.result(r0), srv.result(r3)
    s = bve.BVESphere(seed, level)
    s.init_vorticity(bve.rh54_gaussians(ic_seed, ng, width), ctx, flags=P.FP64)
    torch.cuda.synchronize()
    ref0 = dict(vx=s.physVerts, vzeta=s.relVortVerts, vvel=s.velocityVerts, fx=s.physFaces, fzeta=s.relVortFaces,
                fvel=s.velocityFaces)
    ref0 = {k: v.cpu().numpy() for k, v in ref0.items()}
    for k in KEYS:
        assert _same(init[k], ref0[k]), k
    ctx.rk4_step(s.state(), dt, OMEGA, nsteps, flags=P.FP64)
    torch.cuda.synchronize()
    ref = dict(vx=s.physVerts, vzeta=s.relVortVerts, vvel=s.velocityVerts, fx=s.physFaces, fzeta=s.relVortFaces,
               fvel=s.velocityFaces)
    for k in KEYS:
        assert _same(got[k], ref[k].cpu().numpy()), k


def test_budget_admission_and_cancel():
    torch.cuda.set_device(0)
    one = bve.server_estimate(1, 4)
    with bve.Server(0, budget_bytes=int(one * 1.5)) as srv:
        with pytest.raises(L.LpmError) as e:
            srv.submit(1, 6, 0.0025, 1)
        assert e.value.code == L.LPM_ERR_ADMISSION
        ids = [srv.submit(1, 4, 0.005, 4, ic_seed=s) for s in range(3)]
        last = srv.submit(1, 4, 0.005, 4, ic_seed=99)
        srv.cancel(last)
        assert srv.status(last) == L.REQ_CANCELLED
        with pytest.raises(L.LpmError):
            srv.wait(last, 1.0)
        for rid in ids:
            assert srv.wait(rid, WAIT)
        st = srv.stats()
        assert st["completed"] == 3 and st["cancelled"] == 1 and st["max_running_seen"] == 1
        assert st["reserved_bytes"] == 0
        p50, p99 = srv.latency([0.5, 0.99])
        assert 0 < p50 <= p99
        t = srv.timing(ids[-1])
        assert t["total_s"] >= t["run_s"] > 0 and t["wait_s"] >= 0
        srv.release(ids[0])
        with pytest.raises(L.LpmError):
            srv.result(ids[0])


def test_invalid_requests_rejected():
    torch.cuda.set_device(0)
    with bve.Server(0) as srv:
        for bad in (dict(seed=2, level=3, dt=0.01, nsteps=1), dict(seed=0, level=11, dt=0.01, nsteps=1),
                    dict(seed=0, level=3, dt=float("nan"), nsteps=1), dict(seed=0, level=3, dt=0.01, nsteps=-1),
                    dict(seed=0, level=3, dt=0.01, nsteps=1, n_gaussians=2, gauss_width=0.0)):
            with pytest.raises(L.LpmError) as e:
                srv.submit(**bad)
            assert e.value.code == L.LPM_ERR_INVALID_ARGUMENT
        with pytest.raises(L.LpmError):
            srv.wait(12345, 0.1)
        rid = srv.submit(0, 3, 0.01, 1)
        assert srv.wait(rid, WAIT)
        assert srv.stats()["submitted"] == 1


def test_device_initial_condition_matches_host():
    torch.cuda.set_device(0)
    spec = dict(seed=1, level=4, dt=0.005, nsteps=0, ic_seed=21, n_gaussians=5, gauss_width=0.2)
    out = {}
    for host in (True, False):
        with bve.Server(0, flags=P.FP64, host_ic=host) as srv:
            r0 = srv.submit(**spec)
            r2 = srv.submit(**dict(spec, nsteps=2))
            assert srv.wait(r0, WAIT) and srv.wait(r2, WAIT)
            out[host] = (srv.result(r0), srv.result(r2))
    leaf = bve.build_mesh(1, 4)["fmask"] == 0
    for k, tol in (("vzeta", 1e-13), ("fzeta", 1e-13), ("vvel", 1e-12)):
        a, b = out[True][0][k], out[False][0][k]
        assert np.abs(a - b).max() <= tol * np.abs(a).max(), k
    for k in ("vx", "fx", "fvel"):
        a, b = out[True][1][k], out[False][1][k]
        if k.startswith("f"):
            a, b = a[leaf], b[leaf]
        assert np.abs(a - b).max() <= 1e-10 * np.abs(a).max(), k


def test_tiny_meshes_match_single_solve_path(ctx):
    """Levels 0-2 of both seeds in one server (a work item smaller than a tile, one source
    chunk), FP64 with the host initial condition: each equals BVESphere + lpm_bve_rk4_step."""
    torch.cuda.set_device(0)
    specs = [dict(seed=sd, level=lv, dt=0.01, nsteps=2, ic_seed=30 + 3 * sd + lv, n_gaussians=ng, gauss_width=0.3)
             for sd in (0, 1) for lv, ng in ((0, 0), (1, 2), (2, 64))]
    with bve.Server(0, flags=P.FP64, host_ic=True) as srv:
        ids = [srv.submit(**sp) for sp in specs]
        for rid in ids:
            assert srv.wait(rid, WAIT)
        got = [srv.result(rid) for rid in ids]
    for sp, g in zip(specs, got):
        s = bve.BVESphere(sp["seed"], sp["level"])
        s.init_vorticity(bve.rh54_gaussians(sp["ic_seed"], sp["n_gaussians"], sp["gauss_width"]), ctx, flags=P.FP64)
        ctx.rk4_step(s.state(), sp["dt"], OMEGA, sp["nsteps"], flags=P.FP64)
        torch.cuda.synchronize()
        want = dict(vx=s.physVerts, vzeta=s.relVortVerts, vvel=s.velocityVerts, fx=s.physFaces,
                    fzeta=s.relVortFaces, fvel=s.velocityFaces)
        for k in KEYS:
            assert _same(g[k], want[k].cpu().numpy()), (sp, k)


def test_concurrent_clients():
    """Four client threads submit and wait at the same time; every result equals the same
    request run alone (the C ABI is safe to call from any thread)."""
    import threading
    torch.cuda.set_device(0)
    specs = [dict(seed=(t + k) % 2, level=3 + (t + k) % 2, dt=0.005, nsteps=2 + k, ic_seed=100 * t + k)
             for t in range(4) for k in range(3)]
    alone = [_alone(P.FP32C, sp) for sp in specs]
    got = [None] * len(specs)
    errors = []
    with bve.Server(0, flags=P.FP32C) as srv:
        def client(t):
            try:
                mine = [(i, srv.submit(**specs[i])) for i in range(3 * t, 3 * t + 3)]
                for i, rid in mine:
                    assert srv.wait(rid, WAIT)
                    got[i] = srv.result(rid)
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append(e)
        threads = [threading.Thread(target=client, args=(t,)) for t in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors, errors
        assert srv.stats()["completed"] == len(specs)
    for a, g in zip(alone, got):
        for k in KEYS:
            assert _same(g[k], a[k]), k
