#!/usr/bin/env python
"""Benchmark of the GB300 BVE path: RK4 steps/s on one solve at icosahedral level 7.

Workload (the single-solve configuration the headline metric is quoted on): icosahedral
level 7 (163,842 vertices; 436,900 faces of which 327,680 leaves are the sources), RH54
relative vorticity plus 3 seeded Gaussian vortices (amplitude U(-2,2), width 0.1 rad),
Omega = 2 pi, eps = 0, dt = 0.00125 (0.01 at level 4, halved per level).  A step is one
RK4 step (four direct-sum evaluations over every vertex and face target).  Synthetic data
generated on the host; nothing is downloaded.

Printed JSON line (rank 0):
  value      RK4 steps/s, whole job, device-resident inputs, graph-replayed steps
  e2e        the same through lpm_bve_rk4_step with the state copied host->device before
             and device->host after every step (pinned buffers)
  roofline   pair kernel: algorithmic pairs per launch / CUDA-event launch time, against
             the FP32 FMA-pipe peak (13 FMA-pipe lane-ops per pair)
  cpu_baseline  the CPU oracle (OpenMP restatement of the reference path) on the host cores
  fp64_gpu   the plain FP64 GPU path on a sample of targets, and FP32C-vs-FP64 error there

--impl reference times the reference's CPU path (the oracle port; the reference itself
cannot be built here) on the same workload, each step a bounded sample of targets.
Under torchrun (N > 1) every rank advances its own replica of the solve ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SEED_BASE = 20261203
WORKLOAD = dict(seed_kind=0, level=7, ngauss=3, width=0.1, omega=2 * math.pi, eps=0.0, ic_seed=SEED_BASE + 1)


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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--level", type=int, default=WORKLOAD["level"])
    ap.add_argument("--prec", choices=["fp32c", "fp64"], default="fp32c")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--err-steps", type=int, default=0,
                    help="c2: also advance an FP64 trajectory beside an FP32C one for this many steps and report "
                         "the per-step velocity/vorticity errors (device norms; FP64 is ~150x slower)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU-baseline sample budget")
    ap.add_argument("--config", choices=["c2", "c3", "c4", "c5"], default="c2",
                    help="c2: single solve icos L7 (default, the headline); c3: 64-solve uneven ensemble; "
                         "c4: continuous-batching server under Poisson arrivals; "
                         "c5: icos L8, eps 0.01, 8 vortices, then the stream function at all targets")
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
                    help="c4: a server with LPM_BVE_TREECODE (requests of >= 1e9 pairs per evaluation run on "
                         "its tree-code thread)")
    ap.add_argument("--tree-only", action="store_true",
                    help="c5: time the tree-code leg alone (no direct steps; for profiling the tree path)")
    return ap.parse_args()


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


def workload_desc(level):
    w = dict(WORKLOAD, level=level)
    return (f"icosahedral level {level}, RH54 + {w['ngauss']} Gaussian vortices (seed {w['ic_seed']}, "
            f"amp U(-2,2), width {w['width']}), eps {w['eps']}, dt {time_step(level):g}, Omega 2pi")


def mesh_sizes(level):
    nv = 2 + 10 * 4 ** level
    nl = 20 * 4 ** level
    nall = 20 * (4 ** (level + 1) - 1) // 3
    return nv, nall, nl


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
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
            if gpu_id:
                cmd += ["-i", gpu_id]
            self.fh = open(self.path, "w")
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
        for line in open(self.path):
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
    w = dict(WORKLOAD, level=args.level, dt=time_step(args.level))
    nv, nall, nl = mesh_sizes(args.level)

    t0 = time.time()
    sphere = bve.BVESphere(w["seed_kind"], args.level, omega=w["omega"], layout="left", device=dev)
    ic = bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"])
    sphere.init_vorticity(ic, ctx, flags=prec, eps=w["eps"])
    torch.cuda.synchronize()
    t_init = time.time() - t0
    s0 = clone_sphere(bve, sphere) if not args.no_tree and prec == P.FP32C and rank == 0 else None
    st = sphere.state()

    def barrier():
        if world > 1:
            dist.barrier()

    def rank_max(x):
        return max_over_ranks(x, world, dev)

    # FP32 FMA-pipe peak at the current clock (roofline denominator)
    fma_peak_lane_ops, probes = fma_peak(P, local_rank)

    # warm-up: builds the plan and captures the step graph
    t0 = time.time()
    ctx.rk4_step(st, w["dt"], w["omega"], max(1, args.warmup), flags=prec, eps=w["eps"])
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
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(nsteps):
            flush.zero_()
            ctx.rk4_step(st, w["dt"], w["omega"], 1, flags=prec, eps=w["eps"])
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
    # 1) instrumented pass: per-launch CUDA events around the pair kernel (direct launches)
    el_instr, (pair_ms, pair_n) = timed(args.steps, True)
    # 2) headline pass: graph-replayed steps (the product's default path)
    el_graph, _ = timed(args.steps, False)
    clocks = sampler.stop()
    el_graph_max = rank_max(el_graph)
    el_instr_max = rank_max(el_instr)

    ms_per_step = el_graph_max / args.steps
    value = whole_job_rate(world, args.steps, el_graph_max)
    pairs_alg = (nv + nl) * nl                 # algorithmic pairs per evaluation
    pairs_done = (nv + nall) * nl              # computed (masked parents are targets too)
    pair_avg_ms = pair_ms / max(1, pair_n)
    achieved = pairs_alg / (pair_avg_ms * 1e-3) / 1e9
    peak_at_probe = fma_peak_lane_ops / OPS_PER_PAIR / 1e9
    sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
    peak_nominal = sms * 128 * 2070e6 / OPS_PER_PAIR / 1e9

    # 3) end to end through the public API with host buffers
    names = ("vx", "vzeta", "vvel", "fx", "fzeta", "fvel")
    host = {n: torch.empty(getattr(st, n).shape, dtype=torch.float64, pin_memory=True) for n in names}
    for n in names:
        host[n].copy_(getattr(st, n))
    torch.cuda.synchronize()
    bytes_step = sum(host[n].numel() * 8 for n in names)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.e2e_steps):
        for n in names:
            getattr(st, n).copy_(host[n], non_blocking=True)
        ctx.rk4_step(st, w["dt"], w["omega"], 1, flags=prec, eps=w["eps"])
        for n in names:
            host[n].copy_(getattr(st, n), non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    el_e2e = rank_max(e0.elapsed_time(e1))
    e2e_value = whole_job_rate(world, args.e2e_steps, el_e2e)

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
        "config": {
            "workload": workload_desc(args.level),
            "targets": nv + nall, "sources": nl, "vertices": nv, "faces": nall,
            "pairs_per_eval_algorithmic": pairs_alg, "pairs_per_eval_computed": pairs_done,
            "evals_per_step": 4,
            "l2": "256 MiB buffer written between steps (inside the timed region)",
            "parallelism": f"replicas x{world}",
        },
        "pair_interactions_per_s": world * 4 * pairs_alg / (ms_per_step * 1e-3),
        "instrumented_ms_per_step": el_instr_max / args.steps,
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
            "pair_launch_ms_avg": pair_avg_ms,
            "pair_launches": pair_n,
            "traffic": TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl),
            "traffic_note": "bytes per launch: ncu DRAM read+write of a level-6 launch scaled by targets+sources",
            "algorithmic_bytes": 24 * (nv + nall) + 32 * nl,
            "hbm": hbm_line(TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl), pair_avg_ms),
        },
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": bytes_step,
                "d2h_bytes_per_step": bytes_step, "steps": args.e2e_steps},
        "gpu_launches": 13 * args.steps,
        "init_s": t_init,
        "warmup_s": t_warm,
    }
    if clocks:
        out["clocks"] = clocks

    # 4) plain FP64 GPU path and FP32C accuracy on a target sample (same state)
    if not args.no_fp64 and rank == 0:
        out["fp64_gpu"] = fp64_sample(ctx, sphere, w, P, torch, np, pairs_done, ms_per_step)

    # 4b) the tree code beside the direct sum (approximation; not the headline)
    if s0 is not None:
        tree = tree_leg(P, bve, torch, ctx, s0, w["dt"], w["eps"], args.steps, flush, fma_peak_lane_ops)
        tree["speedup_vs_direct_fp32c"] = tree["rk4_steps_per_s"] / (args.steps / (el_graph * 1e-3))
        out["treecode"] = tree
        del s0

    # 5) CPU baseline (rank 0, single GPU only)
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        out["cpu_baseline"] = cpu_baseline(sphere.state(), sphere, w, args, pairs_done)
    # 6) per-step error of the FP32C trajectory against the FP64 one
    if args.err_steps > 0 and rank == 0:
        out["per_step_error"] = per_step_error(ctx, w, args.level, args.err_steps, dev, P, bve, torch)
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


def per_step_error(ctx, w, level, nsteps, dev, P, bve, torch):
    """FP64 and FP32C trajectories from the same initial state; after every RK4 step the
    relative l2/linf of the FP32C velocity (vertices; leaf faces, area-weighted), relative
    vorticity and face positions against FP64, reduced on the device (lpm_errnorms)."""
    ic = bve.rh54_gaussians(w["ic_seed"], w["ngauss"], w["width"])
    mesh = bve.build_mesh(w["seed_kind"], level)
    runs = {}
    for name, flags in (("fp64", P.FP64), ("fp32c", P.FP32C)):
        s = bve.BVESphere(w["seed_kind"], level, omega=w["omega"], device=dev, mesh=mesh)
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


def fp64_sample(ctx, sphere, w, P, torch, np, pairs_done, ms_per_step, eps=0.0):
    """Plain FP64 GPU path on 8192 sampled vertex targets; FP32C error on the same targets.
    (Vertices: a face centre given as a distinct target would coincide with its own source.)"""
    rng = np.random.default_rng(5)
    leaf = np.flatnonzero(sphere.mesh["fmask"] == 0)
    pts = sphere.physVerts
    idx = torch.from_numpy(rng.choice(pts.shape[0], 8192, replace=False)).to(pts.device)
    tgt = pts[idx].contiguous()
    src = (sphere.physFaces, sphere.relVortFaces, sphere.faces_area, sphere.faces_mask)
    res = {}
    for name, flags in (("fp64", P.FP64), ("fp32c", P.FP32C | P.MESH_TARGETS)):
        ctx.velocity(tgt, *src, flags=flags, eps=eps)  # plan
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        u, _ = ctx.velocity(tgt, *src, flags=flags, eps=eps)
        e1.record()
        torch.cuda.synchronize()
        res[name] = (u.cpu().numpy(), e0.elapsed_time(e1))
    ns = int(leaf.size)
    rate64 = 8192 * ns / (res["fp64"][1] * 1e-3)
    steps64 = rate64 / (4 * pairs_done)
    u64, u32 = res["fp64"][0], res["fp32c"][0]
    err = float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64))
    return {"pairs_per_s": rate64, "steps_per_s_extrapolated": steps64,
            "speedup_fp32c_vs_fp64": (1000.0 / ms_per_step) / steps64,
            "sample": "velocity at 8192 random vertex targets from all leaf sources, one evaluation",
            "fp32c_vs_fp64_velocity_rel_l2": err}


def cpu_baseline(st, sphere, w, args, pairs_done):
    """CPU oracle on the host cores, bounded sample of the same evaluation."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    vx = sphere.physVerts.cpu().numpy(); fx = sphere.physFaces.cpu().numpy()
    z = sphere.relVortFaces.cpu().numpy(); a = sphere.faces_area.cpu().numpy(); m = sphere.mesh["fmask"]
    ns = int((m == 0).sum())
    tg = np.concatenate([vx, fx])
    rng = np.random.default_rng(11)
    n = 256
    t = 0.0
    while True:
        sel = tg[rng.choice(tg.shape[0], n, replace=False)]
        t0 = time.time()
        O.velocity_distinct(sel, fx, z, a, m)
        t = time.time() - t0
        if t > args.cpu_seconds / 4 or n >= tg.shape[0] // 2:
            break
        n = min(tg.shape[0] // 2, int(n * max(2.0, min(8.0, args.cpu_seconds / 4 / max(t, 1e-3)))))
    # final measured sample of ~cpu_seconds
    n = min(tg.shape[0], max(n, int(n * args.cpu_seconds / max(t, 1e-3))))
    sel = tg[rng.choice(tg.shape[0], n, replace=False)]
    t0 = time.time()
    O.velocity_distinct(sel, fx, z, a, m)
    t = time.time() - t0
    rate = n * ns / t
    return {"value": rate / (4 * pairs_done), "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "pairs_per_s": rate,
            "sample": f"FP64 velocity at {n} random targets from all {ns} leaf sources, {t:.1f} s, "
                      f"extrapolated to one RK4 step (4 evaluations of {pairs_done} pairs)"}


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
    ens = ctx.ensemble([s.state() for s in spheres], flags=P.FP32C)
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
                   "autotune": bool(args.autotune)},
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
        "pair_kernel": {"kernel": "treeFP32C<32,8,256,8>", "pairs_per_evaluation": ts["pairs"],
                        "direct_pairs": ts["direct_pairs"], "proxy_pairs": ts["far_pairs"],
                        "computed_pairs_per_s": rate, "frac_of_fma_peak": rate / peak},
    }


def run_large(args, rank, world, local_rank):
    """Config 5: icosahedral level 8 (655,362 vertices, 1,747,620 faces, 1,310,720 sources), RH54 + 8
    Gaussian vortices, eps = 0.01, RK4 steps, then the stream function at all targets."""
    import numpy as np
    import torch

    import lpmkokkos_gb300 as P
    from lpmkokkos_gb300 import bve
    P.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = bve.Context(local_rank, autotune=args.autotune)
    level, eps = 8, 0.01
    dt = time_step(level)
    nv, nall, nl = mesh_sizes(level)
    t0 = time.time()
    s = bve.BVESphere(0, level, device=dev)
    s.init_vorticity(bve.rh54_gaussians(SEED_BASE + 5, 8), ctx, flags=P.FP32C, eps=eps)
    torch.cuda.synchronize()
    t_init = time.time() - t0
    if args.tree_only:
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
        lane_ops, probes = fma_peak(P, local_rank)
        sampler = ClockSampler(gpu_uuid(local_rank))
        ctx.rk4_step(clone_sphere(bve, s).state(), dt, 2 * math.pi, max(1, args.warmup),
                     flags=P.FP32C | P.TREECODE, eps=eps)
        tree = tree_leg(P, bve, torch, ctx, s, dt, eps, args.steps, flush, lane_ops, check_steps=0)
        clocks = sampler.stop()
        if rank == 0:
            print(json.dumps({"metric": "RK4 steps/s (tree code)", "value": tree["rk4_steps_per_s"],
                              "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                              "higher_is_better": True, "dtype": "f32c", "data": "synthetic",
                              "config": {"workload": f"icosahedral level 8, RH54 + 8 Gaussian vortices, eps {eps}, "
                                                     f"dt {dt:g}; tree code only"},
                              "treecode": tree, "probes": probes, "clocks": clocks}), flush=True)
        ctx.close()
        return
    s0 = clone_sphere(bve, s) if not args.no_tree else None
    st = s.state()
    ctx.rk4_step(st, dt, 2 * math.pi, max(1, args.warmup), flags=P.FP32C, eps=eps)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    ctx.set_timing(True); ctx.timing()
    sampler = ClockSampler(gpu_uuid(local_rank))
    el = _timed_region(torch, stream, lambda: ctx.rk4_step(st, dt, 2 * math.pi, 1, flags=P.FP32C, eps=eps),
                       args.steps, flush)
    clocks = sampler.stop()
    pair_ms, pair_n = ctx.timing(); ctx.set_timing(False)
    el = max_over_ranks(el, world, dev)
    # stream function (and velocity) at every vertex and face
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.solve(ctx, flags=P.FP32C, eps=eps, psi=True)
    e1.record(stream)
    torch.cuda.synchronize()
    psi_ms = e0.elapsed_time(e1)
    lane_ops, probes = fma_peak(P, local_rank)
    pairs_alg = (nv + nl) * nl
    achieved = pairs_alg / (pair_ms / pair_n * 1e-3) / 1e9
    peak = lane_ops / OPS_PER_PAIR / 1e9
    fp64 = fp64_sample(ctx, s, dict(WORKLOAD, level=level, dt=dt), P, torch, np, (nv + nall) * nl,
                       el / args.steps, eps=eps)
    tree = None
    if s0 is not None:
        tree = tree_leg(P, bve, torch, ctx, s0, dt, eps, args.steps, flush, lane_ops)
        tree["speedup_vs_direct_fp32c"] = tree["rk4_steps_per_s"] / whole_job_rate(1, args.steps, el)
        tree["speedup_vs_direct_fp64_gpu"] = (tree["rk4_steps_per_s"] / fp64["steps_per_s_extrapolated"]
                                              if fp64 and fp64.get("steps_per_s_extrapolated") else None)
        del s0
    out = {
        "metric": "pair-interactions/s", "value": world * 4 * pairs_alg * args.steps / (el * 1e-3),
        "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps, "rk4_steps_per_s": whole_job_rate(world, args.steps, el),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32c",
        "data": "synthetic (seeded RH54 + 8 Gaussian vortices on a generated icosahedral mesh)",
        "config": {"workload": f"icosahedral level 8, RH54 + 8 Gaussian vortices (seed {SEED_BASE + 5}), "
                               f"eps {eps}, dt {dt:g}, Omega 2pi; stream function at all targets after the steps",
                   "targets": nv + nall, "sources": nl, "autotune": bool(args.autotune)},
        "psi_and_velocity_all_targets_ms": psi_ms,
        "roofline": {"bound": "fp32_fma_pipe", "kernel": "pairFP32C", "achieved": achieved, "peak": peak,
                     "unit": "Gpair/s", "frac": achieved / peak, "pair_launch_ms_avg": pair_ms / pair_n,
                     "peak_source": "FP32 FMA-pipe probe (FFMA / FFMA2, the larger) / 13 lane-ops per pair",
                     "probes": probes, "traffic": TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl),
                     "hbm": hbm_line(TRAFFIC_BYTES_PER_PARTICLE * (nv + nall + nl), pair_ms / pair_n)},
        "fp64_gpu": fp64, "init_s": t_init, "clocks": clocks, "treecode": tree,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


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
    sflags = P.FP32C | (P.TREECODE if args.tree else 0)
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
        **({"computed_pairs_note": "tree-code requests count the direct-sum pairs their evaluations replace"}
           if args.tree else {}),
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
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    O.build()
    w = dict(WORKLOAD, level=args.level)
    m = O.mesh(w["seed_kind"], args.level)
    z = O.rh54_gaussians(m["fx"], w["ic_seed"], w["ngauss"], w["width"])
    nv, nall, nl = mesh_sizes(args.level)
    pairs_done = (nv + nall) * nl
    tg = np.concatenate([m["vx"], m["fx"]])
    rng = np.random.default_rng(3)
    # size one sample to ~3 s of CPU work
    n = 256
    sel = tg[rng.choice(tg.shape[0], n, replace=False)]
    t0 = time.time(); O.velocity_distinct(sel, m["fx"], z, m["farea"], m["fmask"]); t = time.time() - t0
    n = max(256, min(tg.shape[0], int(n * 3.0 / max(t, 1e-3))))
    rates = []
    for k in range(args.warmup + args.steps):
        sel = tg[rng.choice(tg.shape[0], n, replace=False)]
        t0 = time.time()
        O.velocity_distinct(sel, m["fx"], z, m["farea"], m["fmask"])
        t = time.time() - t0
        if k >= args.warmup:
            rates.append(n * nl / t)
    rate = statistics.median(rates)
    steps = rate / (4 * pairs_done)
    sample = (f"each step: FP64 velocity at {n} random vertex/face targets from all {nl} leaf sources, "
              f"extrapolated to one RK4 step (4 evaluations of {pairs_done} pairs)")
    out = {
        "impl": "reference",
        "metric": "RK4 steps/s", "value": steps, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded workload)",
        "config": {"workload": workload_desc(args.level), "targets": nv + nall, "sources": nl,
                   "implementation": "CPU oracle: OpenMP restatement of the reference BVE path "
                                     "(Kokkos reference not buildable: no Kokkos/Trilinos/MPI/VTK)"},
        "pair_interactions_per_s": rate,
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
        {"c2": run_ours, "c3": run_ensemble, "c4": run_server, "c5": run_large}[args.config](args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
