#!/usr/bin/env python
"""Benchmark of the GB300 BVE path: RK4 steps/s of one solve at icosahedral level 8.

Default workload (the largest single-GPU configuration of the headline metric): icosahedral
level 8 -- 655,362 vertices; 1,747,620 faces of which 1,310,720 leaves are the sources -- RH54
relative vorticity plus 8 seeded Gaussian vortices (amplitude U(-2,2), width 0.1 rad),
Omega = 2 pi, eps = 0.01, dt = 0.000625 (0.01 at level 4, halved per level), RK4 steps, then
the stream function and velocity at every vertex and face.  A step is one RK4 step: four
direct-sum evaluations over every vertex and face target (2,403,+ targets x 1,310,720 sources).
Synthetic data generated on the host; nothing is downloaded.  ``--config c2`` runs the
level-7 single solve (RH54 + 3 vortices, eps 0) the same way; it is also reported as a
secondary leg of the default line.

Printed JSON line (rank 0):
  value        RK4 steps/s, whole job, device-resident state, graph-replayed steps
  e2e          the same through lpm_bve_rk4_step with the state copied host->device before and
               device->host after every step (pinned buffers)
  roofline     pair kernel: algorithmic pairs per launch / CUDA-event launch time, against the
               FP32 FMA-pipe peak (13 FMA-pipe lane-ops per pair)
  psi_pass     the closing stream-function + velocity evaluation at every target
  oracle_parity  FP32C and plain-FP64 GPU results against the CPU oracle on 4,096 + 4,096
               sampled vertex / leaf-face targets summed over all sources, initial and final state
  fp64_gpu     the plain FP64 GPU path: its pair rate on a target sample at this level, and a full
               FP64 RK4 step at level 6 timed beside a sample there (the sample's validity)
  cpu_baseline the CPU oracle (OpenMP restatement of the reference path) on the host cores
  c2_level7    the level-7 single solve: steps/s and its pair kernel's roofline fraction

--impl reference times the reference's CPU path (the oracle port; the reference itself cannot
be built here) on the same workload and config: each step is one evaluation over a bounded
random sample of targets, extrapolated to a full RK4 step, and one full evaluation at level 6 is
timed beside a sample there.  Under torchrun (N > 1) every rank advances its own replica of the
solve ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SEED_BASE = 20261203
# single-solve workloads: c2 = icosahedral level 7, c5 = icosahedral level 8 (the default)
WORKLOADS = {
    "c2": dict(seed_kind=0, level=7, ngauss=3, width=0.1, omega=2 * math.pi, eps=0.0, ic_seed=SEED_BASE + 1,
               psi_pass=False),
    "c5": dict(seed_kind=0, level=8, ngauss=8, width=0.1, omega=2 * math.pi, eps=0.01, ic_seed=SEED_BASE + 5,
               psi_pass=True),
}


def time_step(level: int) -> float:
    """dt = 0.01 at level 4 (the CPU-runnable configuration), halved per level: the Courant
    number 2 pi dt / sqrt(4 pi / N_faces) of tests/LpmBVETest.cpp:22 stays at its level-4 value.
    A fixed dt = 0.01 at level 7 moves stage positions ~2 mesh spacings off the sphere, where
    the reference's 1 - x.y denominator crosses zero for nearest neighbours."""
    return 0.01 * 2.0 ** (4 - level)


OPS_PER_PAIR = 13  # FP32 FMA-pipe lane operations per velocity pair in the FP32C kernel
# DRAM bytes per pair-kernel launch per particle (target + source): ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one level-6 launch, 6.91 MB for 150,182 targets + 81,920 sources
# (profiles/pair_fp32c_icos_L6_ncu_full.md).  Traffic follows the O(N) inputs (each source tile
# is re-read from L2, not DRAM), so it scales with targets + sources, not with pairs.
TRAFFIC_BYTES_PER_PARTICLE = 6.91e6 / (150182 + 81920)


def fma_peak(P, device):
    """Achievable FP32 FMA-pipe rate in lane-ops/s at the current clock: the larger of the
    scalar-FFMA and paired-FFMA (f32x2) probes, with both figures."""
    import ctypes
    rates = {}
    for name in ("lpm_probe_fp32_fma", "lpm_probe_fp32_fma2"):
        r, ms = ctypes.c_double(), ctypes.c_double()
        P._lib.check(getattr(P.lib(), name)(device, 200000, ctypes.byref(r), ctypes.byref(ms)))
        rates[name] = r.value
    return max(rates.values()), {"ffma_lane_ops_per_s": rates["lpm_probe_fp32_fma"],
                                 "ffma2_lane_ops_per_s": rates["lpm_probe_fp32_fma2"]}


def measured_peaks():
    """The machine's measured peaks (HBM copy bandwidth, bf16 GEMM) when the file is present."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def hbm_line(traffic_bytes, launch_ms):
    """DRAM bandwidth of the pair kernel against the measured HBM copy peak: shows that the
    kernel is not memory-bound (its traffic follows the O(N) inputs)."""
    peak = measured_peaks().get("hbm_gbs")
    achieved = traffic_bytes / (launch_ms * 1e-3) / 1e9
    return {"achieved_gbs": achieved, "peak_gbs": peak, "frac": (achieved / peak) if peak else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peak else None}


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--prec", choices=["fp32c", "fp64"], default="fp32c")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="RK4 steps of the end-to-end pass (0: as many as --steps, at least 3)")
    ap.add_argument("--err-steps", type=int, default=0,
                    help="c2/c5: also advance an FP64 trajectory beside an FP32C one for this many steps and report "
                         "the per-step velocity/vorticity errors (device norms; FP64 is ~150x slower)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the sampled-target oracle comparison")
    ap.add_argument("--no-secondary", action="store_true", help="c5: skip the level-7 secondary leg")
    ap.add_argument("--no-symmetric", action="store_true",
                    help="steps with the plain pair kernel (LPM_BVE_NO_SYMMETRIC: every leaf pair in both "
                         "directions) instead of the symmetric leaf kernel (c2, c5; c3 ensembles; c4 server)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU-baseline sample budget")
    ap.add_argument("--config", choices=["c2", "c3", "c4", "c5"], default="c5",
                    help="c5: icos L8, eps 0.01, 8 vortices, RK4 steps then the stream function at all targets "
                         "(default, the headline); c2: single solve icos L7; c3: 64-solve uneven ensemble; "
                         "c4: continuous-batching server under Poisson arrivals")
    ap.add_argument("--level", type=int, default=0, help="c2/c5: override the mesh level (0: the config's)")
    ap.add_argument("--requests", type=int, default=96, help="c4: number of requests")
    ap.add_argument("--rate", type=float, default=8.0, help="c4: mean arrivals per second (0: set by --util)")
    ap.add_argument("--util", type=float, default=0.7, help="c4 with --rate 0: target device utilisation")
    ap.add_argument("--req-steps", type=int, default=10, help="c4: RK4 steps per request")
    ap.add_argument("--levels", default="3-7", help="c4: mesh levels, e.g. 3-8")
    ap.add_argument("--level-weights", default=".3,.3,.2,.15,.05",
                    help="c4: comma-separated weights per level (empty: uniform)")
    ap.add_argument("--kinds", choices=["both", "icos"], default="both", help="c4: mesh seeds")
    ap.add_argument("--autotune", action="store_true", help="let the library time launch shapes first")
    ap.add_argument("--no-tree", action="store_true",
                    help="c2/c3/c5: skip the tree-code leg (LPM_BVE_TREECODE, reported beside the direct sum)")
    ap.add_argument("--tree", action="store_true",
                    help="c4: a server with LPM_BVE_TREECODE (requests of >= 1e9 pairs per evaluation are set up "
                         "by its tree threads and stepped in tree classes)")
    ap.add_argument("--tree-only", action="store_true",
                    help="c2/c5: time the tree-code leg alone (no direct steps; for profiling the tree path)")
    return ap.parse_args(argv)


def max_over_ranks(x: float, world: int, device=None) -> float:
    """Maximum of a per-rank scalar (timings: the job is as slow as its slowest replica)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def whole_job_rate(world: int, units_per_rank: int, max_elapsed_ms: float) -> float:
    """Units per second of the whole job: every replica processed units_per_rank units."""
    return world * units_per_rank / (max_elapsed_ms * 1e-3)


def workload(config: str, level: int = 0) -> dict:
    w = dict(WORKLOADS[config])
    if level:
        w["level"] = level
    w["dt"] = time_step(w["level"])
    return w


def workload_desc(w: dict) -> str:
    return (f"icosahedral level {w['level']}, RH54 + {w['ngauss']} Gaussian vortices (seed {w['ic_seed']}, "
            f"amp U(-2,2), width {w['width']}), eps {w['eps']}, dt {w['dt']:g}, Omega 2pi"
            + ("; stream function and velocity at every target after the steps" if w["psi_pass"] else ""))


def mesh_sizes(level):
    nv = 2 + 10 * 4 ** level
    nl = 20 * 4 ** level
    nall = 20 * (4 ** (level + 1) - 1) // 3
    return nv, nall, nl


def bench_config(w: dict, world: int) -> dict:
    """The `config` object of the line: identical in this arm and in the reference arm."""
    nv, nall, nl = mesh_sizes(w["level"])
    return {"workload": workload_desc(w), "targets": nv + nall, "sources": nl, "vertices": nv, "faces": nall,
            "pairs_per_eval_algorithmic": (nv + nl) * nl, "pairs_per_eval_computed": (nv + nall) * nl,
            "evals_per_step": 4, "eps": w["eps"], "dt": w["dt"],
            "l2": "256 MiB buffer written between steps (inside the timed region)",
            "parallelism": f"replicas x{world}"}


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
def gpu_uuid(local_rank):
    """nvidia-smi id of this rank's GPU (its UUID), or None to query every visible GPU."""
    try:
        import torch
        u = str(getattr(torch.cuda.get_device_properties(local_rank), "uuid", ""))
        return ("GPU-" + u) if u and not u.startswith("GPU-") else (u or None)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms into a temporary file while a
    timed region runs; stop() summarises them."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.proc = None
        try:
            fd, self.path = tempfile.mkstemp(prefix="lpm_clocks_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
            if gpu_id:
                cmd += ["-i", gpu_id]
            self.proc = subprocess.Popen(cmd, stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            lines = fh.readlines()
        os.unlink(self.path)
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------------
def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.distributed as dist

    import lpmkokkos_gb300 as P
    from lpmkokkos_gb300 import bve

    P.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = bve.Context(local_rank, autotune=args.autotune)
    prec = P.FP32C if args.prec == "fp32c" else P.FP64
    sflags = prec | (P.NO_SYMMETRIC if args.no_symmetric else 0)  # RK4 step flags
    w = workload(args.config, args.level)
    level, eps = w["level"], w["eps"]
    nv, nall, nl = mesh_sizes(level)

    t0 = time.time()
    sphere = bve.BVESphere(w["seed_kind"], level, omega=w["omega"], layout="left", device=dev)
    ic = bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"])
    sphere.init_vorticity(ic, ctx, flags=prec, eps=eps)
    torch.cuda.synchronize()
    t_init = time.time() - t0
    if args.tree_only:
        return tree_only(args, P, bve, torch, ctx, sphere, w, local_rank)
    s0 = clone_sphere(bve, sphere) if not args.no_tree and prec == P.FP32C and rank == 0 else None
    st = sphere.state()

    def barrier():
        if world > 1:
            dist.barrier()

    def rank_max(x):
        return max_over_ranks(x, world, dev)

    # FP32 FMA-pipe peak at the current clock (roofline denominator)
    fma_peak_lane_ops, probes = fma_peak(P, local_rank)

    # parity of the initial state (FP32C from init_vorticity, FP64 at the sampled targets)
    parity = {}
    if not args.no_parity and rank == 0:
        parity["initial"] = oracle_parity(ctx, P, torch, np, sphere, w, prec, solve=False)

    # warm-up: builds the plan and captures the step graph
    t0 = time.time()
    ctx.rk4_step(st, w["dt"], w["omega"], max(1, args.warmup), flags=sflags, eps=eps)
    torch.cuda.synchronize()
    t_warm = time.time() - t0

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2
    stream = torch.cuda.current_stream()

    def timed(nsteps, instrumented):
        if instrumented:
            ctx.set_timing(True)
            ctx.timing(reset=True)
        barrier()
        torch.cuda.synchronize()
        e0, e1 = _events(torch)
        e0.record(stream)
        for _ in range(nsteps):
            flush.zero_()
            ctx.rk4_step(st, w["dt"], w["omega"], 1, flags=sflags, eps=eps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        el = e0.elapsed_time(e1)
        pair = None
        if instrumented:
            pair = ctx.timing(reset=True)
            ctx.set_timing(False)
        return el, pair

    sampler = ClockSampler(gpu_uuid(local_rank))
    # 1) headline pass: graph-replayed steps (the product's default path)
    el_graph, _ = timed(args.steps, False)
    # 2) instrumented pass: per-launch CUDA events around the pair kernel (direct launches)
    n_instr = max(1, min(args.steps, 2))
    el_instr, (pair_ms, pair_n) = timed(n_instr, True)
    clocks = sampler.stop()
    el_graph_max = rank_max(el_graph)
    el_instr_max = rank_max(el_instr)

    ms_per_step = el_graph_max / args.steps
    value = whole_job_rate(world, args.steps, el_graph_max)
    cfg = bench_config(w, world)
    pairs_alg = cfg["pairs_per_eval_algorithmic"]
    pairs_done = cfg["pairs_per_eval_computed"]
    pair_avg_ms = pair_ms / max(1, pair_n)
    achieved = pairs_alg / (pair_avg_ms * 1e-3) / 1e9
    peak_at_probe = fma_peak_lane_ops / OPS_PER_PAIR / 1e9
    sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    peak_nominal = sms * 128 * 2070e6 / OPS_PER_PAIR / 1e9

    # 3) end to end through the public API with host buffers
    e2e_steps = args.e2e_steps if args.e2e_steps > 0 else max(3, args.steps)
    names = ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")
    host = {n: torch.empty(getattr(st, n).shape, dtype=torch.float64, pin_memory=True) for n in names}
    for n in names:
        host[n].copy_(getattr(st, n))
    torch.cuda.synchronize()
    bytes_step = sum(host[n].numel() * 8 for n in names)
    barrier()
    e0, e1 = _events(torch)
    e0.record(stream)
    for _ in range(e2e_steps):
        for n in names:
            getattr(st, n).copy_(host[n], non_blocking=True)
        ctx.rk4_step(st, w["dt"], w["omega"], 1, flags=sflags, eps=eps)
        for n in names:
            host[n].copy_(getattr(st, n), non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    el_e2e = rank_max(e0.elapsed_time(e1))
    e2e_value = whole_job_rate(world, e2e_steps, el_e2e)
    steps_done = max(1, args.warmup) + args.steps + n_instr + e2e_steps

    out = {
        "metric": "RK4 steps/s",
        "value": value,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32c" if prec == P.FP32C else "f64",
        "data": "synthetic (seeded RH54 + Gaussian vortices on a generated icosahedral mesh)",
        "config": cfg,
        "pair_interactions_per_s": world * 4 * pairs_alg / (ms_per_step * 1e-3),
        "instrumented_ms_per_step": el_instr_max / n_instr,
        "roofline": {
            "bound": "fp32_fma_pipe",
            "kernel": "pairFP32C" if prec == P.FP32C else "pairFP64",
            "achieved": achieved,
            "peak": peak_at_probe,
            "unit": "Gpair/s",
            "frac": achieved / peak_at_probe,
            "peak_source": "FP32 FMA-pipe probe (independent FFMA / FFMA2 chains, the larger, this run) "
                           "/ 13 lane-ops per pair",
            "probes": probes,
            "peak_nominal_2070MHz": peak_nominal,
            "frac_of_nominal": achieved / peak_nominal,
            "frac_computed_pairs": pairs_done / (pair_avg_ms * 1e-3) / 1e9 / peak_at_probe,
            "pair_launch_ms_avg": pair_avg_ms,
            "pair_launches": pair_n,
            "traffic": TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl),
            "traffic_note": "bytes per launch: ncu DRAM read+write of a level-6 launch scaled by targets+sources",
            "algorithmic_bytes": 24 * (nv + nall) + 32 * nl,
            "hbm": hbm_line(TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl), pair_avg_ms),
        },
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": bytes_step,
                "d2h_bytes_per_step": bytes_step, "steps": e2e_steps},
        "gpu_launches": 13 * args.steps,
        "init_s": t_init,
        "warmup_s": t_warm,
    }
    if clocks:
        out["clocks"] = clocks

    # 4) the closing stream-function + velocity evaluation at every target (vertex and face
    #    evaluations; the first call builds their two plans, the second is timed)
    solved = False
    if w["psi_pass"]:
        ms = []
        for _ in range(2):
            e0, e1 = _events(torch)
            e0.record(stream)
            sphere.solve(ctx, flags=prec, eps=eps, psi=True)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(rank_max(e0.elapsed_time(e1)))
        psi_ms = ms[1]
        out["psi_pass"] = {"ms": psi_ms, "first_call_ms": ms[0], "pairs": pairs_done,
                           "computed_pairs_per_s": pairs_done / (psi_ms * 1e-3),
                           "steps_done_before": steps_done,
                           "config5_job_s": (10 * ms_per_step + psi_ms) * 1e-3,
                           "note": "first_call_ms includes building the vertex and face plans; config5_job_s = "
                                   "10 timed RK4 steps + this pass"}
        solved = True
    # 5) parity of the final state against the oracle
    if not args.no_parity and rank == 0:
        parity["final"] = oracle_parity(ctx, P, torch, np, sphere, w, prec, solve=not solved)
        parity["final"]["after_steps"] = steps_done
        out["oracle_parity"] = parity
        out["oracle_rel_l2"] = {"fp32c_u": max(v["fp32c"]["u_l2"] for v in parity.values()),
                                "fp32c_psi": max(v["fp32c"]["psi_l2"] for v in parity.values()),
                                "fp64_u_maxrel": max(v["fp64"]["u_maxrel"] for v in parity.values()),
                                "fp64_psi_maxrel": max(v["fp64"]["psi_maxrel"] for v in parity.values())}

    # 6) plain FP64 GPU path: sample rate here, full step vs sample at level 6
    if not args.no_fp64 and rank == 0:
        out["fp64_gpu"] = fp64_denominators(ctx, P, bve, torch, np, sphere, w, pairs_done, ms_per_step)

    # 7) the tree code beside the direct sum (approximation; not the headline)
    if s0 is not None:
        tree = tree_leg(P, bve, torch, ctx, s0, w["dt"], eps, args.steps, flush, fma_peak_lane_ops,
                        check_steps=1 if level >= 8 else 2)
        tree["speedup_vs_direct_fp32c"] = tree["rk4_steps_per_s"] / (args.steps / (el_graph * 1e-3))
        out["treecode"] = tree
        del s0

    # 8) CPU baseline (rank 0, single GPU only)
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(sphere, args, pairs_done, eps)
    # 9) per-step error of the FP32C trajectory against the FP64 one
    if args.err_steps > 0 and rank == 0:
        out["per_step_error"] = per_step_error(ctx, w, args.err_steps, dev, P, bve, torch)
    # 10) the level-7 single solve as a secondary leg of the level-8 line
    if args.config == "c5" and not args.level and not args.no_secondary and prec == P.FP32C:
        del sphere, st, flush
        ctx.invalidate()
        torch.cuda.empty_cache()
        out["c2_level7"] = secondary_leg(args, ctx, P, bve, torch, dev, world, rank_max, fma_peak_lane_ops)
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


def secondary_leg(args, ctx, P, bve, torch, dev, world, rank_max, lane_ops):
    """Config 2 (icosahedral level 7, RH54 + 3 vortices, eps 0): RK4 steps/s over --steps
    graph-replayed steps after --warmup, and its pair kernel's roofline fraction."""
    w = workload("c2")
    s = bve.BVESphere(w["seed_kind"], w["level"], omega=w["omega"], layout="left", device=dev)
    s.init_vorticity(bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"]), ctx, flags=P.FP32C, eps=w["eps"])
    st = s.state()
    ctx.rk4_step(st, w["dt"], w["omega"], max(1, args.warmup), flags=P.FP32C, eps=w["eps"])
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    fn = lambda: ctx.rk4_step(st, w["dt"], w["omega"], 1, flags=P.FP32C, eps=w["eps"])  # noqa: E731
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    el = rank_max(_timed_region(torch, stream, fn, args.steps, flush))
    ctx.set_timing(True); ctx.timing()
    _timed_region(torch, stream, fn, 2, flush)
    pair_ms, pair_n = ctx.timing(); ctx.set_timing(False)
    cfg = bench_config(w, world)
    achieved = cfg["pairs_per_eval_algorithmic"] / (pair_ms / pair_n * 1e-3)
    peak = lane_ops / OPS_PER_PAIR
    return {"workload": cfg["workload"], "rk4_steps_per_s": whole_job_rate(world, args.steps, el),
            "ms_per_step": el / args.steps, "steps": args.steps,
            "pair_launch_ms_avg": pair_ms / pair_n, "roofline_frac": achieved / peak,
            "pairs_per_eval_algorithmic": cfg["pairs_per_eval_algorithmic"]}


def oracle_parity(ctx, P, torch, np, sphere, w, prec, solve=True):
    """The sphere's velocity and stream function at every target (FP32C; evaluated here when
    `solve`, else as init_vorticity or the stream-function pass left them) and the plain FP64
    path at the sampled targets, against the CPU oracle on 4,096 random vertices and 4,096 random
    leaf faces summed over all sources: relative L2 for FP32C, max |e| / max |ref| for FP64
    (oracle/sampled_parity.py, part of the oracle)."""
    from oracle import sampled_parity as SP
    t0 = time.time()
    eps = w["eps"]
    if solve:
        sphere.solve(ctx, flags=prec, eps=eps, psi=True)
    torch.cuda.synchronize()
    vidx, fidx = SP.sample_targets(sphere.mesh["nverts"], sphere.mesh["fmask"], seed=w["level"])
    vx, fx = sphere.physVerts.cpu().numpy(), sphere.physFaces.cpu().numpy()
    z = sphere.relVortFaces.cpu().numpy()
    got32 = (sphere.velocityVerts.cpu().numpy()[vidx], sphere.streamFnVerts.cpu().numpy()[vidx],
             sphere.velocityFaces.cpu().numpy()[fidx], sphere.streamFnFaces.cpu().numpy()[fidx])
    ref = SP.oracle_at(vx, fx, z, sphere.mesh["farea"], sphere.mesh["fmask"], vidx, fidx, eps=eps)
    got64 = SP.gpu_fp64_at(ctx, P, torch, sphere.physVerts, sphere.physFaces, sphere.relVortFaces,
                           sphere.faces_area, sphere.faces_mask, vidx, fidx, eps=eps)
    return {"fp32c": SP.compare(got32, ref), "fp64": SP.compare(got64, ref),
            "sample": f"{vidx.size} random vertices + {fidx.size} random leaf faces, all "
                      f"{int((sphere.mesh['fmask'] == 0).sum())} sources, velocity and stream function",
            "seconds": time.time() - t0}


def per_step_error(ctx, w, nsteps, dev, P, bve, torch):
    """FP64 and FP32C trajectories from the same initial state; after every RK4 step the
    relative l2/linf of the FP32C velocity (vertices; leaf faces, area-weighted), relative
    vorticity and face positions against FP64, reduced on the device (lpm_errnorms)."""
    ic = bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"])
    mesh = bve.build_mesh(w["seed_kind"], w["level"])
    runs = {}
    for name, flags in (("fp64", P.FP64), ("fp32c", P.FP32C)):
        s = bve.BVESphere(w["seed_kind"], w["level"], omega=w["omega"], device=dev, mesh=mesh)
        s.init_vorticity(ic, ctx, flags=flags, eps=w["eps"])
        runs[name] = s
    a, b = runs["fp64"], runs["fp32c"]
    area, parents = a.faces_area, a.faces_mask

    def norms():
        uv = ctx.errnorms(b.velocityVerts, a.velocityVerts)
        uf = ctx.errnorms(b.velocityFaces, a.velocityFaces, area, parents)
        zf = ctx.errnorms(b.relVortFaces, a.relVortFaces, area, parents, abs_linf=True)
        xf = ctx.errnorms(b.physFaces, a.physFaces, area, parents)
        return {"u_verts_l2": uv[1], "u_verts_linf": uv[2], "u_faces_l2": uf[1], "u_faces_linf": uf[2],
                "zeta_faces_l2": zf[1], "zeta_faces_linf": zf[2], "x_faces_l2": xf[1]}

    rows = [dict(step=0, **norms())]
    t0 = time.time()
    for k in range(1, nsteps + 1):
        ctx.rk4_step(a.state(), w["dt"], w["omega"], 1, flags=P.FP64, eps=w["eps"])
        ctx.rk4_step(b.state(), w["dt"], w["omega"], 1, flags=P.FP32C, eps=w["eps"])
        torch.cuda.synchronize()
        rows.append(dict(step=k, **norms()))
    return {"steps": nsteps, "seconds": time.time() - t0, "rows": rows,
            "max_u_l2": max(max(r["u_verts_l2"], r["u_faces_l2"]) for r in rows),
            "max_zeta_l2": max(r["zeta_faces_l2"] for r in rows),
            "note": "leaf faces area-weighted, masked parent faces skipped; vertices unweighted"}


def _fp64_sample_rate(ctx, P, torch, np, sphere, eps, ntargets=32768, seed=5):
    """Plain FP64 GPU pair rate on ntargets random vertex targets over all leaf sources (one
    evaluation after its plan is built); also returns the FP32C velocity's relative L2 distance
    from FP64 on the same targets.  (Vertices: a face centre given as a distinct target would
    coincide with its own source.)  32,768 targets make 256 tiles x 8 source chunks of work
    items, enough to fill every resident CTA slot: 8,192 targets left slots idle and measured
    16 % below the full-step rate at level 6."""
    rng = np.random.default_rng(seed)
    pts = sphere.physVerts
    idx = torch.from_numpy(rng.choice(pts.shape[0], min(ntargets, pts.shape[0]), replace=False)).to(pts.device)
    tgt = pts[idx].contiguous()
    src = (sphere.physFaces, sphere.relVortFaces, sphere.faces_area, sphere.faces_mask)
    res = {}
    for name, flags in (("fp64", P.FP64), ("fp32c", P.FP32C | P.MESH_TARGETS)):
        ctx.velocity(tgt, *src, flags=flags, eps=eps)  # plan
        torch.cuda.synchronize()
        e0, e1 = _events(torch)
        e0.record()
        u, _ = ctx.velocity(tgt, *src, flags=flags, eps=eps)
        e1.record()
        torch.cuda.synchronize()
        res[name] = (u.cpu().numpy(), e0.elapsed_time(e1))
    ctx.invalidate()
    ns = int((sphere.mesh["fmask"] == 0).sum())
    rate64 = idx.numel() * ns / (res["fp64"][1] * 1e-3)
    u64, u32 = res["fp64"][0], res["fp32c"][0]
    return rate64, float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64))


def fp64_denominators(ctx, P, bve, torch, np, sphere, w, pairs_done, ms_per_step, full_level=6):
    """The plain FP64 GPU path (the GPU oracle of the "FP32C vs FP64" target: at least 4x its RK4 steps/s).
    A full FP64 step at this level takes minutes (level 8: ~12 min), so its steps/s is
    extrapolated from the pair rate on 32,768 sampled vertex targets; the extrapolation is checked
    by one full FP64 RK4 step at level `full_level` (graph-replayed, after a warm-up step) timed
    beside the same kind of sample at that level."""
    rate, err32 = _fp64_sample_rate(ctx, P, torch, np, sphere, w["eps"])
    steps64 = rate / (4 * pairs_done)
    wf = dict(w, level=full_level, dt=time_step(full_level))
    s = bve.BVESphere(0, full_level, omega=w["omega"], layout="left", device=sphere.physVerts.device)
    s.init_vorticity(bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"]), ctx, flags=P.FP32C, eps=w["eps"])
    st = s.state()
    ctx.rk4_step(st, wf["dt"], w["omega"], 1, flags=P.FP64, eps=w["eps"])  # plan + captured graph
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = _events(torch)
    e0.record(stream)
    ctx.rk4_step(st, wf["dt"], w["omega"], 1, flags=P.FP64, eps=w["eps"])
    e1.record(stream)
    torch.cuda.synchronize()
    full_ms = e0.elapsed_time(e1)
    nv6, nall6, nl6 = mesh_sizes(full_level)
    full_rate = 4 * (nv6 + nall6) * nl6 / (full_ms * 1e-3)
    rate6, _ = _fp64_sample_rate(ctx, P, torch, np, s, w["eps"])
    ctx.invalidate()
    return {"pairs_per_s": rate, "steps_per_s_extrapolated": steps64,
            "speedup_fp32c_vs_fp64": (1000.0 / ms_per_step) / steps64,
            "sample": "velocity at 32768 random vertex targets from all leaf sources, one evaluation",
            "fp32c_vs_fp64_velocity_rel_l2": err32,
            "full_step_check": {"level": full_level, "fp64_rk4_step_ms": full_ms,
                                "computed_pairs_per_s": full_rate, "sample_pairs_per_s": rate6,
                                "sample_over_full": rate6 / full_rate}}


def cpu_baseline(sphere, args, pairs_done, eps):
    """CPU oracle on the host cores, bounded sample of the same evaluation."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    vx = sphere.physVerts.cpu().numpy(); fx = sphere.physFaces.cpu().numpy()
    z = sphere.relVortFaces.cpu().numpy(); a = sphere.faces_area.cpu().numpy(); m = sphere.mesh["fmask"]
    ns = int((m == 0).sum())
    tg = np.concatenate([vx, fx[m == 0]])
    rng = np.random.default_rng(11)
    n = 256
    t = 0.0
    while True:
        sel = tg[rng.choice(tg.shape[0], n, replace=False)]
        t0 = time.time()
        O.velocity_distinct(sel, fx, z, a, m, eps=eps)
        t = time.time() - t0
        if t > args.cpu_seconds / 4 or n >= tg.shape[0] // 2:
            break
        n = min(tg.shape[0] // 2, int(n * max(2.0, min(8.0, args.cpu_seconds / 4 / max(t, 1e-3)))))
    # final measured sample of ~cpu_seconds
    n = min(tg.shape[0], max(n, int(n * args.cpu_seconds / max(t, 1e-3))))
    sel = tg[rng.choice(tg.shape[0], n, replace=False)]
    t0 = time.time()
    O.velocity_distinct(sel, fx, z, a, m, eps=eps)
    t = time.time() - t0
    rate = n * ns / t
    return {"value": rate / (4 * pairs_done), "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "pairs_per_s": rate,
            "sample": f"FP64 velocity at {n} random vertex / leaf-face points from all {ns} leaf sources, {t:.1f} s, "
                      f"extrapolated to one RK4 step (4 evaluations of {pairs_done} pairs)"}


def tree_only(args, P, bve, torch, ctx, s, w, local_rank):
    """--tree-only: the tree-code leg alone on this workload (profiling the tree path)."""
    dev = s.physVerts.device
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    lane_ops, probes = fma_peak(P, local_rank)
    sampler = ClockSampler(gpu_uuid(local_rank))
    ctx.rk4_step(clone_sphere(bve, s).state(), w["dt"], w["omega"], max(1, args.warmup),
                 flags=P.FP32C | P.TREECODE, eps=w["eps"])
    tree = tree_leg(P, bve, torch, ctx, s, w["dt"], w["eps"], args.steps, flush, lane_ops, check_steps=0)
    clocks = sampler.stop()
    print(json.dumps({"metric": "RK4 steps/s (tree code)", "value": tree["rk4_steps_per_s"], "unit": "steps/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                      "dtype": "f32c", "data": "synthetic",
                      "config": {"workload": workload_desc(w) + "; tree code only"},
                      "treecode": tree, "probes": probes, "clocks": clocks}), flush=True)
    ctx.close()


# ------------------------------------------------------------------------------------------
# further configurations (not the default line)
# ------------------------------------------------------------------------------------------
def courant_dt(seed_kind: int, level: int) -> float:
    """dt at the Courant number 2 pi dt / sqrt(4 pi / N_faces) of icosahedral level 4, dt = 0.01."""
    nf = (20 * (4 ** (level + 1) - 1) // 3) if seed_kind == 0 else 2 * (4 ** (level + 1) - 1)
    nf4 = 20 * (4 ** 5 - 1) // 3
    return 0.01 * math.sqrt(nf4 / nf)


def _timed_region(torch, stream, fn, nsteps, flush):
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(nsteps):
        flush.zero_()
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_ensemble(args, rank, world, local_rank):
    """Config 3: 64 independent solves, levels drawn uniformly from icosahedral and cubed-sphere
    levels 4-7, RH54 + 3 seeded Gaussian vortices each, FP32C, one persistent pair launch per RK4
    evaluation for all solves, graph-captured steps."""
    import numpy as np
    import torch

    import lpmkokkos_gb300 as P
    from lpmkokkos_gb300 import bve
    P.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = bve.Context(local_rank, autotune=args.autotune)
    rng = np.random.default_rng(SEED_BASE + 3)
    menu = [(0, 4), (0, 5), (0, 6), (0, 7), (1, 4), (1, 5), (1, 6), (1, 7)]
    picks = [menu[i] for i in rng.integers(0, len(menu), size=64)]
    meshes, spheres = {}, []
    t0 = time.time()
    for m, (sk, lv) in enumerate(picks):
        if (sk, lv) not in meshes:
            meshes[(sk, lv)] = bve.build_mesh(sk, lv)
        s = bve.BVESphere(sk, lv, device=dev, mesh=meshes[(sk, lv)])
        s.init_vorticity(bve.rh54_gaussians(SEED_BASE + 3 + 1000 * m, 3), ctx, flags=P.FP32C)
        spheres.append(s)
    torch.cuda.synchronize()
    t_init = time.time() - t0
    dts = [courant_dt(sk, lv) for sk, lv in picks]
    oms = [2 * math.pi] * len(picks)
    initial = [clone_sphere(bve, s) for s in spheres] if not args.no_tree else None
    eflags = P.FP32C | (P.NO_SYMMETRIC if args.no_symmetric else 0)
    ens = ctx.ensemble([s.state() for s in spheres], flags=eflags)
    info = ens.info()
    ens.step(dts, oms, max(1, args.warmup))
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    sampler = ClockSampler(gpu_uuid(local_rank))
    el = max_over_ranks(_timed_region(torch, stream, lambda: ens.step(dts, oms, 1), args.steps, flush), world, dev)
    clocks = sampler.stop()
    steps_per_s = whole_job_rate(world, args.steps, el)
    alg = 0
    for sk, lv in picks:
        nv = 2 + (10 if sk == 0 else 6) * 4 ** lv
        nl = (20 if sk == 0 else 6) * 4 ** lv
        alg += (nv + nl) * nl
    finite = all(bool(torch.isfinite(s.velocityVerts).all()) for s in spheres)
    out = {
        "metric": "ensemble RK4 steps/s", "value": steps_per_s, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32c",
        "data": "synthetic (seeded RH54 + Gaussian vortices, 64 generated meshes)",
        "config": {"workload": "64 solves, levels uniform over icosahedral 4-7 and cubed sphere 4-7 "
                               f"(seed {SEED_BASE + 3}), dt at the level-4 Courant number, FP32C",
                   "levels": {f"{'icos' if k[0] == 0 else 'cube'}{k[1]}": picks.count(k) for k in menu},
                   "work_items": info["nitems"], "grid": info["grid"], "device_bytes": info["device_bytes"],
                   "autotune": bool(args.autotune), "symmetric_leaf_kernel": not args.no_symmetric},
        "pair_interactions_per_s": world * 4 * alg * args.steps / (el * 1e-3),
        "computed_pairs_per_s": world * 4 * info["pairs_per_eval"] * args.steps / (el * 1e-3),
        "gpu_launches": 13 * args.steps, "init_s": t_init, "all_vertex_velocities_finite": finite,
        "clocks": clocks,
    }
    ens.close()
    if initial is not None:
        # the same ensemble with the tree code (each solve its own octree and lists; an
        # approximation outside the reference, beside the direct numbers), from the initial states
        tens = ctx.ensemble([s.state() for s in initial], flags=P.FP32C | P.TREECODE)
        tens.step(dts, oms, 1)
        torch.cuda.synchronize()
        el_t = max_over_ranks(_timed_region(torch, stream, lambda: tens.step(dts, oms, 1), args.steps, flush), world, dev)
        tens.close()
        out["treecode"] = {"ensemble_rk4_steps_per_s": whole_job_rate(world, args.steps, el_t),
                           "ms_per_step": el_t / args.steps,
                           "speedup_vs_direct_ensemble": whole_job_rate(world, args.steps, el_t) / steps_per_s,
                           "params": {"degree": 8, "theta": 0.6, "leaf_points": 512, "min_pairs": 1e9},
                           "note": "solves under 1e9 pairs share one direct launch; the others take one "
                                   "tree-code evaluation each, one after another"}
        del initial
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


def clone_sphere(bve, s):
    """A second BVESphere on the same mesh holding a copy of s's evolving state."""
    c = bve.BVESphere(s.seed, s.level, mesh=s.mesh, device=s.physVerts.device)
    for name in ("physVerts", "relVortVerts", "velocityVerts", "physFaces", "relVortFaces", "velocityFaces"):
        getattr(c, name).copy_(getattr(s, name))
    return c


def tree_leg(P, bve, torch, ctx, s0, dt, eps, steps, flush, lane_ops, check_steps=2):
    """The tree code (LPM_BVE_TREECODE: far clusters through chart-interpolated proxies; an
    approximation outside the reference, reported beside the direct-sum numbers, never in their
    place) on the same workload, from copies of the initial state s0: its distance from the FP32C
    direct sum after `check_steps` RK4 steps, then RK4 steps/s over `steps` timed steps with the
    phase times, the gathered pair kernel's rate and its fraction of the FMA-pipe peak."""
    omega = 2 * math.pi
    b = clone_sphere(bve, s0)
    leaf = torch.from_numpy(s0.mesh["fmask"] == 0).to(s0.physVerts.device)
    errs = None
    if check_steps > 0:
        a = clone_sphere(bve, s0)
        ctx.rk4_step(a.state(), dt, omega, check_steps, flags=P.FP32C, eps=eps)
        ctx.rk4_step(b.state(), dt, omega, check_steps, flags=P.FP32C | P.TREECODE, eps=eps)
        torch.cuda.synchronize()
        rel = lambda x, y: (torch.linalg.norm(x - y) / torch.linalg.norm(y)).item()
        errs = {"velocity_vertices": rel(b.velocityVerts, a.velocityVerts),
                "velocity_leaves": rel(b.velocityFaces[leaf], a.velocityFaces[leaf]),
                "vorticity_vertices": rel(b.relVortVerts, a.relVortVerts),
                "positions_vertices": rel(b.physVerts, a.physVerts)}
        del a
    stream = torch.cuda.current_stream()
    st = b.state()
    el = _timed_region(torch, stream, lambda: ctx.rk4_step(st, dt, omega, 1, flags=P.FP32C | P.TREECODE, eps=eps),
                       steps, flush)
    ctx.set_timing(True); ctx.timing()
    ctx.rk4_step(st, dt, omega, 1, flags=P.FP32C | P.TREECODE, eps=eps)
    torch.cuda.synchronize()
    pair_ms, pair_n = ctx.timing(); ctx.set_timing(False)
    ts = ctx.tree_stats()  # the last of the step's four evaluations
    nv, nf, nl = b.physVerts.shape[0], b.physFaces.shape[0], int(leaf.sum())
    peak = lane_ops / OPS_PER_PAIR
    rate = ts["pairs"] / (pair_ms / pair_n * 1e-3)
    return {
        "rk4_steps_per_s": steps / (el * 1e-3), "ms_per_step": el / steps,
        "params": {"degree": 8, "theta": 0.6, "leaf_points": 512, "min_pairs": 1e9},
        "rel_l2_vs_fp32c_direct_after_steps": check_steps, "rel_l2_vs_fp32c_direct": errs,
        "work_fraction_of_direct_pairs": ts["pairs"] / ((nv + nf) * nl),
        "octree": {"depth": ts["depth"], "nodes": ts["nodes"], "far_clusters": ts["far_clusters"]},
        "phase_ms_per_evaluation": {"octree_build": ts["build_ms"], "upward_pass": ts["upward_ms"],
                                    "interaction_lists": ts["list_ms"], "pair_kernel": pair_ms / pair_n},
        "pair_kernel": {"kernel": "treeFP32C<32,4,128,12>", "pairs_per_evaluation": ts["pairs"],
                        "direct_pairs": ts["direct_pairs"], "proxy_pairs": ts["far_pairs"],
                        "computed_pairs_per_s": rate, "frac_of_fma_peak": rate / peak},
    }


COMPUTED_PAIR_RATE = 2.2e12  # FP32C pairs/s incl. masked-parent targets (measured, icos L7)


def computed_pairs(seed_kind: int, level: int) -> int:
    """Target-source pairs one evaluation computes: (vertices + all faces) x leaf faces."""
    f0, v0 = (20, 10) if seed_kind == 0 else (6, 6)
    nv = 2 + v0 * 4 ** level
    nall = f0 * (4 ** (level + 1) - 1) // 3
    return (nv + nall) * f0 * 4 ** level


def run_server(args, rank, world, local_rank):
    """Config 4: the continuous-batching server under Poisson arrivals.  Each request draws a
    mesh seed (icosahedral, or icosahedral/cubed sphere with equal odds) and a level from
    --levels (--level-weights), RH54 + 3 seeded Gaussian vortices, dt at the level-4 Courant
    number, --req-steps RK4 steps.  The arrival rate is --rate, or with --rate 0 the rate that
    loads the device to --util by the expected service time.  Latency is submit-to-result on the
    host clock: host preparation, upload, queueing, the steps and the copy back are all inside.
    Beside it: the same requests served one at a time by the plain FP64 GPU path, extrapolated
    from its pair rate measured in this run."""
    import threading

    import numpy as np
    import torch

    import lpmkokkos_gb300 as P
    from lpmkokkos_gb300 import bve
    P.build()
    torch.cuda.set_device(local_rank)
    rng = np.random.default_rng(SEED_BASE + 4)
    lo, hi = (int(v) for v in args.levels.split("-"))
    levels = list(range(lo, hi + 1))
    weights = [float(v) for v in args.level_weights.split(",")] if args.level_weights else []
    if len(weights) != len(levels):
        weights = [1.0] * len(levels)
    weights = np.asarray(weights) / np.sum(weights)
    n = args.requests
    kinds = np.zeros(n, dtype=int) if args.kinds == "icos" else rng.integers(0, 2, size=n)
    lvls = rng.choice(levels, size=n, p=weights)
    exp_service = sum(wt * args.req_steps * 4 * np.mean([computed_pairs(k, lv) for k in
                                                          ((0,) if args.kinds == "icos" else (0, 1))])
                      for lv, wt in zip(levels, weights)) / COMPUTED_PAIR_RATE
    rate = args.rate if args.rate > 0 else args.util / exp_service
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    specs = [dict(seed=int(k), level=int(lv), dt=courant_dt(int(k), int(lv)), nsteps=args.req_steps,
                  ic_seed=SEED_BASE + 4 + i) for i, (k, lv) in enumerate(zip(kinds, lvls))]
    sflags = P.FP32C | (P.TREECODE if args.tree else 0) | (P.NO_SYMMETRIC if args.no_symmetric else 0)
    srv = bve.Server(local_rank, flags=sflags)
    # warm-up: one zero-step request per mesh (fills the host mesh/plan cache, loads kernels)
    meshes = sorted({(s["seed"], s["level"]) for s in specs})
    warm = [srv.submit(seed=k, level=lv, dt=0.01, nsteps=0) for k, lv in meshes]
    warm += [srv.submit(seed=0, level=4, dt=0.005, nsteps=2, ic_seed=s) for s in range(max(1, args.warmup))]
    for rid in warm:
        assert srv.wait(rid, 600.0)
        srv.release(rid)
    base = srv.stats()
    ids = [None] * n

    def feeder():
        t0 = time.perf_counter()
        for i, sp in enumerate(specs):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids[i] = srv.submit(**sp)

    sampler = ClockSampler(gpu_uuid(local_rank))
    t_start = time.perf_counter()
    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    for rid in ids:
        assert srv.wait(rid, 7200.0)
    wall = time.perf_counter() - t_start
    clocks = sampler.stop()
    st = srv.stats()
    lat = np.array([srv.timing(r)["total_s"] for r in ids])
    waits = np.array([srv.timing(r)["wait_s"] for r in ids])
    by_level = {}
    for lv in levels:
        sel = lat[lvls == lv]
        if sel.size:
            by_level[str(lv)] = {"n": int(sel.size), "p50_s": float(np.percentile(sel, 50)),
                                 "max_s": float(sel.max())}
    # the same request alone gives the same bits as in the mix
    check = [i for i in range(n) if specs[i]["level"] <= 5][:2]
    mixed = [srv.result(ids[i]) for i in check]
    srv.close()
    same = True
    with bve.Server(local_rank, flags=sflags) as alone:
        for i, got in zip(check, mixed):
            rid = alone.submit(**specs[i])
            assert alone.wait(rid, 600.0)
            ref = alone.result(rid)
            same &= all(np.array_equal(got[k], ref[k], equal_nan=True) for k in ref)
    # plain FP64 GPU path, one request after another: its pair rate on a level-6 sample
    ctx = bve.Context(local_rank)
    s6 = bve.BVESphere(0, 6)
    s6.init_vorticity(bve.rh54_gaussians(SEED_BASE + 4, 3), ctx, flags=P.FP32C)
    tgt = s6.physVerts[:8192].contiguous()
    src = (s6.physFaces, s6.relVortFaces, s6.faces_area, s6.faces_mask)
    ctx.velocity(tgt, *src, flags=P.FP64)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    ctx.velocity(tgt, *src, flags=P.FP64)
    e1.record()
    torch.cuda.synchronize()
    r64 = 8192 * int((s6.mesh["fmask"] == 0).sum()) / (e0.elapsed_time(e1) * 1e-3)
    ctx.close()
    serial64 = sum((sp["nsteps"] * 4 + 1) * computed_pairs(sp["seed"], sp["level"]) for sp in specs) / r64
    solve_steps = st["solve_steps"] - base["solve_steps"]
    pairs = st["pairs"] - base["pairs"]
    tree_equiv = st["tree_equiv_pairs"] - base["tree_equiv_pairs"]
    nearest = lambda q: float(np.sort(lat)[max(0, math.ceil(q * n) - 1)])  # noqa: E731
    kinds_desc = "icosahedral" if args.kinds == "icos" else "icosahedral or cubed sphere"
    out = {
        "metric": "server requests/s", "value": n / wall, "unit": "requests/s", "n_gpus": 1,
        "steps": args.req_steps, "warmup": len(warm), "ms_per_step": None, "higher_is_better": True,
        "scaling": "replicas only", "vs_baseline": None, "dtype": "f32c",
        "data": "synthetic (seeded RH54 + Gaussian vortices on generated meshes, Poisson arrivals)",
        "config": {"workload": f"{n} requests, Poisson arrivals at {rate:.4g}/s, {kinds_desc} levels "
                               f"{lo}-{hi} (weights {', '.join(f'{v:.3g}' for v in weights)}), "
                               f"{args.req_steps} RK4 steps each, dt at the level-4 Courant number, FP32C "
                               f"(seed {SEED_BASE + 4})" + ("; tree-code server" if args.tree else ""),
                   "levels": {str(lv): int((lvls == lv).sum()) for lv in levels},
                   "expected_service_s": exp_service, "offered_utilisation": rate * exp_service},
        "latency_s": {"p50": nearest(0.5), "p99": nearest(0.99), "max": float(lat.max()),
                      "mean_wait": float(waits.mean())},
        "latency_by_level": by_level,
        "solve_steps_per_s": solve_steps / wall, "computed_pairs_per_s": pairs / wall,
        **({"tree_equivalent_pairs_per_s": tree_equiv / wall,
            "tree_equivalent_pairs_note": "tree-code requests: the direct-sum pairs their evaluations replace "
                                          "(work equivalent, not computed)"} if args.tree else {}),
        "server_iterations": st["steps_run"] - base["steps_run"], "max_running": st["max_running_seen"],
        "wall_s": wall, "mix_equals_alone": bool(same), "clocks": clocks,
        "serial_fp64_gpu": {"pairs_per_s": r64, "seconds": serial64, "requests_per_s": n / serial64,
                            "speedup": (n / wall) / (n / serial64),
                            "how": "each request alone on the plain FP64 GPU path: (4 evaluations per step + 1 "
                                   "initial) x computed pairs / FP64 pair rate measured here (level 6)"},
        "e2e": {"value": n / wall, "unit": "requests/s", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------------------
# reference arm: the reference path's CPU implementation (oracle port) on the host cores
# ------------------------------------------------------------------------------------------
def run_reference(args, rank, world):
    """The reference path's CPU implementation (the oracle port: the reference needs Kokkos /
    Trilinos, MPI and VTK, none of which exist here) on all host cores, on the same workload and
    `config` as our arm.  A full evaluation at level 8 takes ~10 min on 16 cores, so each step is
    one FP64 evaluation at a bounded random sample of vertex / face targets over all sources
    (~3 s), extrapolated to a full RK4 step (4 evaluations); one full evaluation at level 6 is
    timed beside a sample there to show the extrapolation holds."""
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    O.build()
    w = workload(args.config if args.config in ("c2", "c5") else "c5", args.level)
    eps = w["eps"]
    m = O.mesh(w["seed_kind"], w["level"])
    z = O.rh54_gaussians(m["fx"], w["ic_seed"], w["ngauss"], w["width"])
    cfg = bench_config(w, world)
    nl, pairs_done = cfg["sources"], cfg["pairs_per_eval_computed"]
    tg = np.concatenate([m["vx"], m["fx"]])
    rng = np.random.default_rng(3)

    def sample_rate(mesh, zz, targets, n):
        sel = targets[rng.choice(targets.shape[0], n, replace=False)]
        t0 = time.time()
        O.velocity_distinct(sel, mesh["fx"], zz, mesh["farea"], mesh["fmask"], eps=eps)
        return n * int((mesh["fmask"] == 0).sum()) / (time.time() - t0)

    # size one sample to ~3 s of CPU work
    n = 256
    r = sample_rate(m, z, tg, n)
    n = max(256, min(tg.shape[0], int(3.0 * r / nl)))
    rates = []
    for k in range(args.warmup + args.steps):
        rk = sample_rate(m, z, tg, n)
        if k >= args.warmup:
            rates.append(rk)
    rate = statistics.median(rates)
    steps = rate / (4 * pairs_done)
    # the extrapolation checked: one full evaluation at level 6 (or the workload's, if lower)
    # beside a sample there
    lf = min(6, w["level"])
    mf = O.mesh(0, lf)
    zf = O.rh54_gaussians(mf["fx"], w["ic_seed"], w["ngauss"], w["width"])
    t0 = time.time()
    O.velocity(mf["vx"], mf["fx"], zf, mf["farea"], mf["fmask"], eps=eps)
    full_s = time.time() - t0
    nvf, nallf, nlf = mesh_sizes(lf)
    full_rate = (nvf + nallf) * nlf / full_s
    tgf = np.concatenate([mf["vx"], mf["fx"]])
    ratef = sample_rate(mf, zf, tgf, min(tgf.shape[0], max(256, int(3.0 * rate / nlf))))
    sample = (f"each step: FP64 velocity at {n} random vertex / face targets from all {nl} leaf sources, "
              f"extrapolated to one RK4 step (4 evaluations of {pairs_done} pairs)")
    out = {
        "impl": "reference",
        "metric": "RK4 steps/s", "value": steps, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded workload)",
        "config": cfg,
        "steps_kind": "sampled evaluations (each extrapolated to one RK4 step)",
        "implementation": "CPU oracle: OpenMP restatement of the reference BVE path (the Kokkos reference is not "
                          "buildable here: no Kokkos/Trilinos/MPI/VTK)",
        "pair_interactions_per_s": rate,
        "full_evaluation_check": {"level": lf, "seconds": full_s, "pairs_per_s": full_rate,
                                  "sample_pairs_per_s": ratef, "sample_over_full": ratef / full_rate},
        "cpu_baseline": {"value": steps, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": steps, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local_rank)
        dist.init_process_group(backend=backend)
    try:
        {"c2": run_ours, "c3": run_ensemble, "c4": run_server, "c5": run_ours}[args.config](args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
