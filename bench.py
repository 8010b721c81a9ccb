#!/usr/bin/env python
"""Benchmark: <Map^3> triplets/s over a Latin-hypercube batch of cosmologies.

Workload (the batched configuration): cosmologies from a seeded Latin
hypercube (Om in [0.2,0.4], sigma8 in [0.7,0.9], h in [0.6,0.8],
w in [-1.2,-0.8], ns in [0.92,1.0], Ob=0.048, z_max=3), source
n(z) ~ z^2 exp(-(z/0.5)^1.5), 10 log-spaced aperture radii 1..32 arcmin ->
220 triplets per cosmology; every (cosmology, triplet) is one adaptive
<Map^3> integral at relative tolerance 1e-4 (the reference's MapMapMap
settings, l in [1, 10/theta_min]). One step = one batch of C cosmologies: the
GPU table build (set_cosmology) plus all C*220 integrals in the FP32
integrand. Inputs are synthetic (no data files are read).

--impl reference times the CPU FP64 restatement of the reference (the
oracle; the reference itself does not build on this machine) on the host
cores, one integral per step, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Map3 triplets/s at <=1e-3 rel err vs FP64: surrogate+FP32 vs plain FP64, 1 GB300"
ARCMIN = 2.9088820866e-4
LHS_SEED = 20261203
N_LHS = 4096
# DRAM bytes (read + write) of one k_map3<float> launch per integral, from
# ncu dram__bytes_read.sum + dram__bytes_write.sum of a 880-integral launch
# (4 LHS cosmologies x 220 triplets: 65.9 + 221.5 MB); the region-store
# traffic grows with the number of integrals
TRAFFIC_PER_INTEGRAL = (70.184192e6 + 225.050112e6) / 880
SFU_PER_NODE = 22  # SFU ops (ex2/rcp.approx) per line-of-sight node of the FP32 BiHalofit evaluation (NF_* rows, merged reciprocals)
NNODE = 96


def lhs_cosmologies(n=N_LHS, seed=LHS_SEED):
    """Latin hypercube: per dimension a random permutation of n strata plus a
    uniform jitter inside each stratum (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    box = [("om", 0.2, 0.4), ("sigma8", 0.7, 0.9), ("h", 0.6, 0.8), ("w", -1.2, -0.8), ("ns", 0.92, 1.0)]
    cols = {}
    for name, lo, hi in box:
        u = (rng.permutation(n) + rng.uniform(size=n)) / n
        cols[name] = lo + u * (hi - lo)
    out = []
    for i in range(n):
        om = float(cols["om"][i])
        out.append(dict(h=float(cols["h"][i]), sigma8=float(cols["sigma8"][i]), omb=0.048, omc=om - 0.048,
                        ns=float(cols["ns"][i]), w=float(cols["w"][i]), om=om, ow=1 - om, zmax=3.0))
    return out


def thetas_220():
    radii = np.exp(np.linspace(np.log(1.0), np.log(32.0), 10)) * ARCMIN
    t = []
    for i in range(10):
        for j in range(i, 10):
            for k in range(j, 10):
                t.append((radii[i], radii[j], radii[k]))
    return np.array(t)


def nz_config():
    zs = np.arange(3001) * 1e-3
    ns = zs ** 2 * np.exp(-(zs / 0.5) ** 1.5)
    return zs, ns


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    import threepoint_gb300 as tp
    from threepoint_gb300.shard import shard_range

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    # two contexts (own stream, tables and region stores) take alternate
    # batches: one batch's table build and launch tail overlap the other's
    # integrals. --no-pipeline runs every step alone on one context.
    nctx = 1 if args.no_pipeline else 2
    ctxs = [tp.Context(local) for _ in range(nctx)]
    for c in ctxs:
        c.set_limits(args.region_cap)
        c.set_map3_cluster(args.map3_cluster)
    ctx = ctxs[0]
    streams = [torch.cuda.ExternalStream(c.stream_handle, device=local) for c in ctxs]
    stream = streams[0]
    cosmos_all = lhs_cosmologies()
    zs, ns = nz_config()
    nz = tp.rebin_n_of_z(zs, ns, 256, 3.0)
    th = thetas_220()
    C = args.cosmo_per_step
    nt = len(th)
    nj = C * nt
    dev = torch.device("cuda", local)
    job_cosmo = torch.arange(C, dtype=torch.int32, device=dev).repeat_interleave(nt)
    job_theta = torch.tensor(np.tile(th, (C, 1)), dtype=torch.float64, device=dev)

    def buffers():
        o = torch.zeros(nj, dtype=torch.float64, device=dev)
        return dict(out=o, err=torch.zeros_like(o), nev=torch.zeros(nj, dtype=torch.int64, device=dev),
                    nlive=torch.zeros(nj, dtype=torch.int64, device=dev),
                    status=torch.zeros(nj, dtype=torch.int32, device=dev))

    bufs = [buffers() for _ in ctxs]
    out, err, nev, nlive, status = (bufs[0][k] for k in ("out", "err", "nev", "nlive", "status"))
    lmax = 0.0 if args.lmax == "ref" else float(args.lmax)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > 129 MB L2

    # each rank walks through its own contiguous block of the LHS (weak scaling,
    # no communication on the data path)
    lo, hi = shard_range(N_LHS, rank, world)

    def cosmo_batch(step):
        off = lo + (step * C) % max(1, hi - lo - C + 1)
        return [tp.cosmology(**c) for c in (cosmos_all * 2)[off:off + C]]

    order = [None]

    def one_step(step, k, timing=None, flush_first=False):
        """Batch `step` on context k: L2 flush (optional), table build, all
        C x 220 integrals; all on context k's stream."""
        c, st, b = ctxs[k], streams[k], bufs[k]
        batch = cosmo_batch(step)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        with torch.cuda.stream(st):
            ev[0].record(st)
            c.set_cosmologies(batch, nz)
            if flush_first:
                flush.zero_()  # L2 flush before the step's integrals (on this step's stream)
            ev[1].record(st)
            c.map3_jobs_device(job_cosmo, job_theta, b["out"], b["err"], b["nev"], b["status"], lMax=lmax,
                               rel_tol=1e-4, precision=tp.FP32, nlive=b["nlive"], job_order=order[0])
            ev[2].record(st)
        if timing is not None:
            timing.append(ev)

    # warm-up; after the first warm-up step the jobs are ordered longest-first
    # by the per-triplet cost seen there (what tp_map3_batch does internally)
    for s in range(args.warmup):
        one_step(s, s % nctx)
        if s == 0 and not args.no_order:
            torch.cuda.synchronize()
            cost = nev.view(C, nt).double().mean(0)
            trip_order = torch.argsort(cost, descending=True)
            order[0] = (torch.arange(C, device=dev).view(C, 1) * nt + trip_order.view(1, nt)).t().reshape(-1)
            order[0] = order[0].to(torch.int32).contiguous()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    start = torch.cuda.Event(enable_timing=True)
    start.record(streams[0])
    for st in streams[1:]:
        st.wait_event(start)
    bad = 0
    for s in range(args.steps):
        one_step(args.warmup + s, s % nctx, flush_first=True)
        if nctx == 1:
            torch.cuda.synchronize()
    ends = []
    for st in streams:
        e = torch.cuda.Event(enable_timing=True)
        e.record(st)
        ends.append(e)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    tot_ms = max(start.elapsed_time(e) for e in ends)
    for b in bufs:
        bad += int((b["status"] != 0).sum().item())
    if bad:
        print(f"warning: {bad} integrals hit a cap in the last steps", file=sys.stderr)
    if dist:
        tt = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tot_ms = float(tt.item())

    # kernel time for the roofline: k_map3 launches timed alone (no overlap),
    # outside the timed region
    timings = []
    live_total = 0
    neval_total = 0
    n_roof = min(args.steps, 3)
    for s in range(n_roof):
        torch.cuda.synchronize()
        one_step(args.warmup + s, 0, timings, flush_first=True)
        torch.cuda.synchronize()
        live_total += int(nlive.sum().item())
        neval_total += int(nev.sum().item())
        if args.dump_costs and s == 0:
            np.savez(args.dump_costs, theta=np.tile(th, (C, 1)), neval=nev.cpu().numpy(), nlive=nlive.cpu().numpy(),
                     value=out.cpu().numpy())
    map3_ms = [t[1].elapsed_time(t[2]) for t in timings]
    build_ms = [t[0].elapsed_time(t[1]) for t in timings]
    integrals = nj * args.steps * world
    value = integrals / (tot_ms * 1e-3)

    # accuracy and the plain FP64 method, outside the timed region: all 220
    # triplets at the four corners of the Latin-hypercube box (every output of
    # those cosmologies, FP32 against the plain FP64 GPU method), timed like
    # `value` (table build + integrals on the device, CUDA events)
    check = corner_cosmologies()[:C]
    ncheck = len(check) * nt
    acc = None
    fp64_val = None
    if not args.no_fp64_plain:
        vals = {}
        for prec in (tp.FP64, tp.FP32):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e[0].record(stream)
                ctx.set_cosmologies([tp.cosmology(**c) for c in check], nz)
                ctx.map3_jobs_device(job_cosmo[:ncheck], job_theta[:ncheck], out[:ncheck], err[:ncheck],
                                     nev[:ncheck], status[:ncheck], lMax=lmax, rel_tol=1e-4, precision=prec)
                e[1].record(stream)
            torch.cuda.synchronize()
            vals[prec] = (out[:ncheck].cpu().numpy().copy(), e[0].elapsed_time(e[1]) * 1e-3,
                          int((status[:ncheck] != 0).sum().item()))
        v64, t64, cap64 = vals[tp.FP64]
        v32, _, cap32 = vals[tp.FP32]
        acc = output_errors(v32, v64)
        acc.update({"cosmologies": "4 corners of the LHS box (Om, sigma8, h, w, ns at their bounds)",
                    "integrals_at_cap_fp64": cap64, "integrals_at_cap_fp32": cap32})
        fp64_val = ncheck / t64

    # e2e: the public host API (host inputs, host outputs) for the same steps
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        ctx.set_cosmologies(cosmo_batch(args.warmup + s), nz)
        res = ctx.map3_batch(th, precision=tp.FP32, check=False)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_val = nj * e2e_steps / e2e_s
    h2d = C * 72 + 256 * 8 + nj * (3 * 8 + 4)
    d2h = nj * (8 + 8 + 8 + 4)

    # roofline of the dominant kernel (k_map3<float>): SFU ops of the live points
    sfu_peak, f32_peak, f64_peak = tp.pipe_peaks(local)
    live_per_launch = live_total / n_roof
    map3_avg_s = statistics.mean(map3_ms) * 1e-3
    achieved = live_per_launch * NNODE * SFU_PER_NODE / map3_avg_s

    if dist:
        dist.barrier()
    if rank != 0:
        return None
    res = {
        "metric": METRIC,
        "value": value,
        "unit": "triplets/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": tot_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{C} LHS cosmologies x 220 theta-triplets per step (4096-cosmology LHS batch)",
                   "cosmologies_per_step": C, "triplets": nt, "rel_tol": 1e-4,
                   "l_range": "[1, 10/theta_min]" if lmax == 0 else f"[1, {lmax:g}]",
                   "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}",
                   "pipeline": "1 context" if nctx == 1 else
                   "2 contexts on 2 streams, alternate batches (table build and launch tail overlap)",
                   "table_build_ms_alone": statistics.mean(build_ms), "map3_ms_alone": statistics.mean(map3_ms),
                   "job_order": "none" if args.no_order else "longest-first by warm-up cost per triplet",
                   "integrand": "FP32 line-of-sight BiHalofit (96 nodes, packed pairs) at every point; "
                                "the b_kappa surrogate network is not used in this line"},
        "e2e": {"value": e2e_val, "unit": "triplets/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "accuracy_fp32_vs_fp64": acc,
        "integrals_at_cap": bad,
        "gpu_launches": 10 * args.steps,  # 9 table-build kernels + k_map3 per step
        "roofline": {"bound": "sfu", "achieved": achieved / 1e9, "peak": sfu_peak / 1e9, "unit": "Gop/s",
                     "frac": achieved / sfu_peak, "traffic": TRAFFIC_PER_INTEGRAL * nj,
                     "traffic_unit": "bytes per launch (ncu, 880-integral capture scaled by integrals)",
                     "peak_source": "measured now by tp_pipe_peaks (ex2.approx.f32 loop, whole device)",
                     "kernel": "k_map3<float>", "kernel_ms_per_launch": map3_avg_s * 1e3,
                     "fp32_peak_tflops": 2 * f32_peak / 1e12, "fp64_peak_tflops": 2 * f64_peak / 1e12,
                     "fma_peaks_source": "tp_pipe_peaks FMA/s x 2 FLOP"},
        "reference_work_equivalent": reference_work(neval_total / n_roof, map3_avg_s),
        "clocks": clocks,
        "plain_fp64_gpu": None if fp64_val is None else {
            "value": fp64_val, "unit": "triplets/s", "integrals": ncheck, "fp32_speedup": value / fp64_val,
            "note": "plain FP64 method (FP64 BiHalofit integrand), table build + integrals on the device "
                    "as in `value`, one batch of the 4 box-corner cosmologies x 220 triplets"},
        "wall_s": wall,
    }
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(args, sample_triplets=args.cpu_sample)
    return res


def corner_cosmologies():
    """Four corners of the Latin-hypercube box: the extremes of Omega_m,
    sigma_8, h, w and n_s, paired so that each parameter takes both bounds."""
    out = []
    for om, s8, h, w, ns in ((0.2, 0.7, 0.6, -1.2, 0.92), (0.4, 0.9, 0.8, -0.8, 1.0),
                             (0.2, 0.9, 0.8, -0.8, 0.92), (0.4, 0.7, 0.6, -1.2, 1.0)):
        out.append(dict(h=h, sigma8=s8, omb=0.048, omc=om - 0.048, ns=ns, w=w, om=om, ow=1 - om, zmax=3.0))
    return out


def output_errors(v32, v64):
    """Per-output relative error of the FP32 integrals against FP64. Outputs
    whose FP64 value is exactly 0 (triplets whose first rule has an all-zero
    filter product, as in the reference) must be 0 in FP32 too."""
    nzm = v64 != 0
    r = np.abs(v32[nzm] - v64[nzm]) / np.abs(v64[nzm])
    return {"outputs": int(v64.size), "nonzero_outputs": int(nzm.sum()),
            "zero_valued_agree": bool(np.array_equal(v32 == 0, v64 == 0)),
            "max_rel": float(r.max()) if r.size else 0.0, "median_rel": float(np.median(r)) if r.size else 0.0,
            "p99_rel": float(np.percentile(r, 99)) if r.size else 0.0,
            "outputs_above_1e-3": int((r > 1e-3).sum())}


def reference_work(points_per_launch, launch_s):
    """The launch's work in operations of the reference's FP64 formula chain:
    evaluated cubature points x the counted operations of one point
    (roofline.json, oracle/opcount.py; transcendental calls weighted as stated
    there). The GPU path folds most of that chain into per-cosmology tables, so
    this rate measures useful work, not the GPU's own instruction rate."""
    try:
        with open(os.path.join(ROOT, "roofline.json")) as f:
            per_point = float(json.load(f)["map3_point"]["flop_equivalent"])
    except (OSError, KeyError, ValueError):
        return None
    return {"flop_equivalent_per_point": per_point, "points_per_launch": points_per_launch,
            "tflop_equivalent_per_s": points_per_launch * per_point / launch_s / 1e12,
            "source": "roofline.json (oracle/opcount.py)",
            "note": "work of the reference's FP64 formula chain per second, not a roofline: the GPU path "
                    "evaluates far fewer operations per point (per-cosmology node tables)"}


def cpu_baseline(args, sample_triplets=2):
    """The CPU FP64 restatement on the host cores, a bounded sample of the
    same workload: the first LHS cosmology, sample_triplets triplets."""
    import oracle

    n = os.cpu_count() or 1
    oracle.set_threads(n)
    c = lhs_cosmologies()[0]
    zs, ns = nz_config()
    nz = oracle.read_n_of_z(zs, ns, 256, 3.0)
    th = thetas_220()
    pick = [th[i] for i in np.linspace(0, len(th) - 1, sample_triplets).astype(int)]
    t0 = time.perf_counter()
    T = oracle.Tables(c, nz)
    for t in pick:
        T.map3(list(t))
    dt = time.perf_counter() - t0
    return {"value": len(pick) / dt, "unit": "triplets/s", "cores": n, "kind": "port",
            "sample": f"{len(pick)} triplets of LHS cosmology 0 incl. its table build, FP64, {n} threads"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    import oracle

    n = os.cpu_count() or 1
    oracle.set_threads(n)
    cos = lhs_cosmologies()
    zs, ns = nz_config()
    nz = oracle.read_n_of_z(zs, ns, 256, 3.0)
    th = thetas_220()
    T = oracle.Tables(cos[0], nz)
    # one integral per step, stepping through the 220 triplets with a stride
    order = [int(i) for i in np.linspace(0, len(th) - 1, args.steps + args.warmup)]
    for s in range(args.warmup):
        T.map3(list(th[order[s]]))
    times = []
    for s in range(args.steps):
        t0 = time.perf_counter()
        T.map3(list(th[order[args.warmup + s]]))
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = args.steps / tot
    return {
        "metric": METRIC, "value": value, "unit": "triplets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": "1 (cosmology, theta-triplet) integral per step of the 4096-LHS x 220 batch",
                   "rel_tol": 1e-4, "l_range": "[1, 10/theta_min]"},
        "cpu_baseline": {"value": value, "unit": "triplets/s", "cores": n, "kind": "port",
                         "sample": f"{args.steps} integrals of LHS cosmology 0 (FP64 CPU restatement, {n} threads)"},
        "e2e": {"value": value, "unit": "triplets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


COSMO_FID = dict(h=0.7, sigma8=0.8, omb=0.048, omc=0.3 - 0.048, ns=0.96, w=-1.0, om=0.3, ow=0.7, zmax=3.0)


def _rel_stats(a, b):
    """per-output relative differences |a-b|/|b| over outputs with |b| > 0"""
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    m = np.abs(b) > 0
    r = np.abs(a[m] - b[m]) / np.abs(b[m])
    return {"max": float(r.max()) if r.size else None, "median": float(np.median(r)) if r.size else None,
            "outputs": int(m.sum())}


def run_gamma(args):
    """Shear 3PCF on the (r, u, v) grid of calculateGamma: 10 log r bins on
    0.1-100', 10 u bins on [0, 1], 10 v bins on [-1, 1] (bin centres), all four
    natural components, centroid convention; FP32 integrand timed, FP64 on a
    subset for the per-output error."""
    import torch

    import threepoint_gb300 as tp

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    ctx = tp.Context(local)
    if args.gamma_region_cap != 32768:
        ctx.set_limits(args.gamma_region_cap)
    zs, ns = nz_config()
    ctx.set_cosmology(tp.cosmology(**COSMO_FID), tp.rebin_n_of_z(zs, ns, 256, 3.0))
    cfg = tp.configGamma(10, 10, 10, 0.0, 1.0, -1.0, 1.0, 0.1, 100.0)
    x, ruv = cfg.triangles()
    n = len(x) if args.gamma_triangles <= 0 else min(len(x), args.gamma_triangles)
    x, ruv = x[:n], ruv[:n]
    ctx.gamma_batch(x[: min(n, 8)], precision=tp.FP32)  # warm-up
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g32 = ctx.gamma_batch(x, precision=tp.FP32, check=False)
        times.append(time.perf_counter() - t0)
        st32 = ctx.last_gamma_status.copy()
        capped = int((st32 != 0).sum())
    sub = np.arange(0, n, max(1, n // args.gamma_fp64_sample))
    t0 = time.perf_counter()
    # the FP64 check runs at the context's cap without escalation (bounded
    # time); its capped triangles are left out of the error statistics
    ctx.set_escalation(0)
    g64 = ctx.gamma_batch(x[sub], precision=tp.FP64, check=False)
    t64 = time.perf_counter() - t0
    st64 = ctx.last_gamma_status.copy()
    ok = st64 == 0
    err = _rel_stats(np.stack([g32[sub][ok].real, g32[sub][ok].imag]), np.stack([g64[ok].real, g64[ok].imag]))
    tot = sum(times)
    return {"metric": "Gamma_0..3 triangles/s (4 natural components, rel. tol 1e-3)", "value": n * args.steps / tot,
            "unit": "triangles/s", "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": tot / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"calculateGamma grid: {n} (r,u,v) bin centres x 4 components, fiducial cosmology",
                       "timing": "host API tp_gamma_batch per step (host inputs and outputs)",
                       "region_cap": args.gamma_region_cap,
                       "escalation": "integrals at the cap integrated again with 16x the cap, up to 2^24 regions",
                       "triangles_at_cap": capped,
                       "capped_r_u_v": [[round(float(v), 4) for v in ruv[i]] for i in np.nonzero(st32)[0][:200]]},
            "fp64": {"triangles": int(len(sub)), "triangles_per_s": len(sub) / t64,
                     "triangles_at_cap": int((st64 != 0).sum()),
                     "note": "FP64 at the region cap without escalation; capped triangles left out of the errors",
                     "rel_err_fp32_vs_fp64": err}}


def run_cov(args):
    """<Map^3> covariance T1 + T2 (square 10x10 deg^2 window) and T4 (infinite
    geometry with the survey area) for a seeded sample of the 24310 (triplet,
    triplet) pairs of the 220 triplets; sigma_eps 0.3, n_gal 10 arcmin^-2.
    Integrals that reach the region cap are counted, not fatal."""
    import torch

    import threepoint_gb300 as tp

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    ctx = tp.Context(local)
    if args.cov_region_cap > 0:
        ctx.set_limits(args.cov_region_cap)
    zs, ns = nz_config()
    ctx.set_shape_noise(0.3, 10 / ARCMIN ** 2, False)
    ctx.set_cosmology(tp.cosmology(**COSMO_FID), tp.rebin_n_of_z(zs, ns, 256, 3.0))
    th = thetas_220()
    pairs = [(i, j) for i in range(len(th)) for j in range(i, len(th))]
    rng = np.random.default_rng(LHS_SEED)
    pick = rng.choice(len(pairs), size=min(args.cov_pairs, len(pairs)), replace=False)
    A = np.array([th[pairs[k][0]] for k in pick])
    B = np.array([th[pairs[k][1]] for k in pick])
    deg = 0.017453
    kw = dict(thetaMax=10 * deg, area=100 * deg * deg)
    all_terms = {"T1": (1, tp.GEOM_SQUARE), "T2": (2, tp.GEOM_SQUARE), "T4": (4, tp.GEOM_INFINITE)}
    terms = tuple((n, *all_terms[n]) for n in args.cov_terms.split(","))
    res, t, capped = {}, {}, {}
    for name, term, geom in terms:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res[name] = ctx.cov_total(term, A, B, geometry=geom, precision=tp.FP32, check=False, **kw)
        t[name] = time.perf_counter() - t0
        capped[name] = ctx.last_capped
    n64 = min(len(pick), args.cov_fp64_pairs)
    err, t64 = {}, {}
    for name, term, geom in terms:
        if name not in args.cov_fp64_terms.split(","):
            continue
        t0 = time.perf_counter()
        r64 = ctx.cov_total(term, A[:n64], B[:n64], geometry=geom, precision=tp.FP64, check=False, **kw)
        t64[name] = time.perf_counter() - t0
        err[name] = _rel_stats(res[name][:n64], r64)
    tot = sum(t.values())
    return {"metric": f"<Map^3> covariance entries/s ({args.cov_terms}; T1, T2 square 10x10 deg^2, T4 infinite with area)",
            "value": len(pick) / tot, "unit": "entries/s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": tot * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{len(pick)} of the 24310 triplet pairs of 220 triplets (seeded sample)",
                       "seconds_per_term": t, "timing": "host API tp_cov_total_batch",
                       "integrals_at_region_cap": capped},
            "fp64": {"pairs": n64, "seconds_per_term": t64, "rel_err_fp32_vs_fp64": err}}


def run_halo(args):
    """Halo-model covariance terms (T5, T7 infinite survey with the 100 deg^2
    area; T6 the square 10x10 deg^2 window) for a seeded sample of the 24310
    triplet pairs of the 220 triplets; sigma_eps 0.3, n_gal 10 arcmin^-2. The
    FP32 node path is timed through the host API; FP64 reruns a few pairs for
    the per-output difference; the CPU oracle integrates the first distinct
    integral of each term on the host cores (a bounded sample: 5-30 s)."""
    import torch

    import threepoint_gb300 as tp

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    ctx = tp.Context(local)
    zs, ns = nz_config()
    nz = tp.rebin_n_of_z(zs, ns, 256, 3.0)
    sig, ngal = 0.3, 10 / ARCMIN ** 2
    ctx.set_shape_noise(sig, ngal, False)
    ctx.set_cosmology(tp.cosmology(**COSMO_FID), nz)
    th = thetas_220()
    pairs = [(i, j) for i in range(len(th)) for j in range(i, len(th))]
    rng = np.random.default_rng(LHS_SEED)
    pick = rng.choice(len(pairs), size=min(args.halo_pairs, len(pairs)), replace=False)
    A = np.array([th[pairs[k][0]] for k in pick])
    B = np.array([th[pairs[k][1]] for k in pick])
    deg = 0.017453
    kw = dict(thetaMax=10 * deg, area=100 * deg * deg)
    all_terms = {"T5": (5, tp.GEOM_INFINITE), "T6": (6, tp.GEOM_SQUARE), "T7": (7, tp.GEOM_INFINITE)}
    terms = tuple((n, *all_terms[n]) for n in args.halo_terms.split(","))
    ctx.halo_tables()  # table build outside the timed region
    res, t, capped = {}, {}, {}
    for name, term, geom in terms:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res[name] = ctx.cov_total(term, A, B, geometry=geom, precision=tp.FP32, check=False, **kw)
        t[name] = time.perf_counter() - t0
        capped[name] = ctx.last_capped
    n64 = min(len(pick), args.halo_fp64_pairs)
    err, t64 = {}, {}
    for name, term, geom in terms:
        if n64 == 0 or name not in args.halo_fp64_terms.split(","):
            continue
        t0 = time.perf_counter()
        r64 = ctx.cov_total(term, A[:n64], B[:n64], geometry=geom, precision=tp.FP64, check=False, **kw)
        t64[name] = time.perf_counter() - t0
        err[name] = _rel_stats(res[name][:n64], r64)
    ctx.close()
    tot = sum(t.values())
    cpu = None
    if not args.no_cpu_baseline and args.halo_cpu_terms:
        import oracle as O

        O.set_threads(0)
        T = O.Tables(COSMO_FID, nz)
        T.set_noise(sig, ngal, False)
        cpu_s, cpu_terms = 0.0, []
        for name in args.halo_cpu_terms.split(","):
            term, geom = all_terms[name]
            mult_idx = O.halo_total_terms(term, A[0], B[0])
            src = list(A[0]) + list(B[0])
            th6 = [src[i] for i in mult_idx[0][1]]
            par = O.CovParams(geom, kw["thetaMax"], kw["area"], 0.0)
            t0 = time.perf_counter()
            T.cov_T_halo(term, par, th6)
            cpu_s += time.perf_counter() - t0
            cpu_terms.append(name)
        cpu = {"value": len(cpu_terms) / cpu_s, "unit": "integrals/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"the first integral of the first pair for {','.join(cpu_terms)} at the reference's "
                         f"tolerances (FP64 oracle, {os.cpu_count()} threads)"}
    return {"metric": f"<Map^3> covariance halo-model entries/s ({args.halo_terms}; T5, T7 infinite with the "
                      f"100 deg^2 area, T6 square 10x10 deg^2)",
            "value": len(pick) / tot, "unit": "entries/s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": tot * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{len(pick)} of the 24310 triplet pairs of 220 triplets (seeded sample)",
                       "seconds_per_term": t, "timing": "host API tp_cov_total_batch",
                       "integrals_at_region_cap": capped},
            "fp64": {"pairs": n64, "seconds_per_term": t64, "rel_err_fp32_vs_fp64": err},
            "cpu_baseline": cpu}


def run_plain(args):
    """The plain form (FP64 BiHalofit, FP64 cubature) on the fiducial
    cosmology and the 20 triplets of radii {2, 4, 8, 16}', through the host
    API, at the reference's l bound [1, 10/theta_min] and at the configuration's
    [1, 1e5]; the FP32 path beside it, and the CPU oracle on a sample of the
    same triplets."""
    import torch

    import threepoint_gb300 as tp

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    zs, ns = nz_config()
    nz = tp.rebin_n_of_z(zs, ns, 256, 3.0)
    ctx = tp.Context(local)
    ctx.set_cosmology(tp.cosmology(**COSMO_FID), nz)
    r = np.array([2.0, 4.0, 8.0, 16.0]) * ARCMIN
    th = np.array([(r[i], r[j], r[k]) for i in range(4) for j in range(i, 4) for k in range(j, 4)])
    out = {}
    vals = {}
    for name, prec in (("fp64", tp.FP64), ("fp32", tp.FP32)):
        for lname, lmax in (("l_ref", 0.0), ("l_1e5", 1e5)):
            ctx.map3_batch(th[:1], precision=prec, lMax=lmax, check=False)  # warm-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            v = ctx.map3_batch(th, precision=prec, lMax=lmax, check=False)
            dt = time.perf_counter() - t0
            vals[(name, lname)] = v[0]
            out[f"{name}_{lname}"] = {"value": len(th) / dt, "unit": "triplets/s", "seconds": dt}
    ctx.close()
    for lname in ("l_ref", "l_1e5"):
        a, b = vals[("fp32", lname)], vals[("fp64", lname)]
        nzm = b != 0
        out[f"fp32_{lname}"]["max_rel_err_vs_fp64"] = float(np.max(np.abs(a[nzm] - b[nzm]) / np.abs(b[nzm])))
    a64, b64 = vals[("fp64", "l_1e5")], vals[("fp64", "l_ref")]
    both = (a64 != 0) & (b64 != 0)
    l_study = {"triplets_zero_at_l_1e5_only": int(((a64 == 0) & (b64 != 0)).sum()),
               "max_rel_shift_where_both_nonzero": float(np.max(np.abs(a64[both] / b64[both] - 1))) if both.any()
               else None,
               "theta_arcmin": (th / ARCMIN).round(3).tolist(), "fp64_l_ref": b64.tolist(), "fp64_l_1e5": a64.tolist(),
               "note": "at [1, 1e5] the first Genz-Malik rule of a large-radius triplet has an all-zero filter "
                       "product (the product underflows at every one of its 33 points), so the cubature stops "
                       "after one region with value 0, as the reference's hcubature_v does"}
    l_shift = vals[("fp64", "l_1e5")] / vals[("fp64", "l_ref")] - 1.0
    res = {"metric": "plain <Map^3> FP64 triplets/s (fiducial cosmology, 20 triplets of {2,4,8,16} arcmin)",
           "value": out["fp64_l_ref"]["value"], "unit": "triplets/s", "n_gpus": 1, "steps": 1, "warmup": 1,
           "ms_per_step": out["fp64_l_ref"]["seconds"] * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "fiducial flat wCDM, n(z) ~ z^2 exp(-(z/0.5)^1.5), 20 triplets, rel 1e-4",
                      "timing": "host API tp_map3_batch (copies included)"},
           "lines": out, "fp64_l_1e5_vs_l_ref_max_rel": float(np.max(np.abs(l_shift[np.isfinite(l_shift)]))),
           "l_range_study": l_study}
    if not args.no_cpu_baseline:
        import oracle

        n = os.cpu_count() or 1
        oracle.set_threads(n)
        T = oracle.Tables(COSMO_FID, oracle.read_n_of_z(zs, ns, 256, 3.0))
        pick = th[:: max(1, len(th) // 2)][:2]
        t0 = time.perf_counter()
        for t in pick:
            T.map3(list(t))
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": len(pick) / dt, "unit": "triplets/s", "cores": n, "kind": "port",
                               "sample": f"{len(pick)} of the 20 triplets, FP64, {n} threads, l in [1, 10/theta_min]"}
    return res


def apm_catalogue(n_gal, fieldsize, seed=7):
    """Seeded synthetic shear catalogue: uniform positions on the field,
    shears = a smooth large-scale pattern + shape noise sigma_eps = 0.3."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, fieldsize, n_gal)
    y = rng.uniform(0.0, fieldsize, n_gal)
    g = 0.02 * np.exp(2j * np.pi * (x / 37.0 + y / 53.0)) + \
        0.3 * (rng.standard_normal(n_gal) + 1j * rng.standard_normal(n_gal)) / np.sqrt(2)
    return x, y, g


def run_apm(args):
    """The measurement side (python_scripts/aperture_mass_computer.py
    extract_Map3): a shear catalogue of n_gal = 10 arcmin^-2 over a
    240' x 240' field, CIC onto 4096^2 pixels, aperture-mass maps for
    theta in {2, 4, 8, 16}' (exponential filter) and <Map^3> of the 20
    triplets. One step = one field. `value` times the device-resident
    pipeline (catalogue already in HBM), `e2e` the host API with the
    catalogue copied in and the 20 values copied out every step."""
    import torch

    import threepoint_gb300 as tp
    from threepoint_gb300 import aperture_mass as G

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    npix, fs, thetas = args.apm_npix, 240.0, [2.0, 4.0, 8.0, 16.0]
    n_gal = int(10 * fs * fs)
    x, y, g = apm_catalogue(n_gal, fs)
    ctx = tp.Context(local)
    plan = G._Plan(ctx, npix, fs, thetas, False)
    dev = torch.device("cuda", local)
    dx, dy = torch.tensor(x, device=dev), torch.tensor(y, device=dev)
    d1, d2 = torch.tensor(g.real.copy(), device=dev), torch.tensor(g.imag.copy(), device=dev)
    ntrip = len(thetas) * (len(thetas) + 1) * (len(thetas) + 2) // 6
    out = torch.zeros(ntrip, dtype=torch.float64, device=dev)
    st = torch.cuda.ExternalStream(ctx.stream_handle, device=local)
    L = tp.lib()

    def step():
        rc = L.tp_apm_extract_map3_device(plan._h, dx.data_ptr(), dy.data_ptr(), d1.data_ptr(), d2.data_ptr(), n_gal,
                                          1, out.data_ptr())
        if rc:
            raise RuntimeError(L.tp_last_error(ctx._h).decode())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    t_dev = e0.elapsed_time(e1) * 1e-3
    gpu_vals = out.cpu().numpy()
    # e2e: host catalogue in, host results out, every step
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 5))):
        host = plan.extract_map3(x, y, g, True)
    e2e_s = (time.perf_counter() - t0) / max(1, min(args.steps, 5))
    res = {"metric": "<Map^3> fields/s (FFT aperture-mass measurement, extract_Map3)", "value": args.steps / t_dev,
           "unit": "fields/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{n_gal} galaxies on a 240' field, CIC to {npix}^2, theta {thetas}', "
                                  f"exponential filter, 20 triplets, same border for all",
                      "fft_size": int(L.tp_apm_fft_size(plan._h)),
                      "l2": "working set of several GB per field (> L2)"},
           "e2e": {"value": 1.0 / e2e_s, "unit": "fields/s", "h2d_bytes_per_step": 4 * 8 * n_gal,
                   "d2h_bytes_per_step": 8 * ntrip},
           "gpu_launches": (6 + 2 * len(thetas)) * args.steps, "gpu_launches_note": "this library's kernels; cuFFT's transforms (3 + 2 per aperture per step) in addition", "clocks": clocks,
           "device_vs_host_api_max_rel": float(np.max(np.abs(host - gpu_vals)) / np.max(np.abs(gpu_vals)))}
    # the same pipeline with FP32 transforms and Fourier products (gridding,
    # maps and sums FP64), device-resident, against the FP64 values
    plan32 = G._Plan(ctx, npix, fs, thetas, False, precision=tp.FP32)
    out32 = torch.zeros_like(out)

    def step32():
        rc = L.tp_apm_extract_map3_device(plan32._h, dx.data_ptr(), dy.data_ptr(), d1.data_ptr(), d2.data_ptr(),
                                          n_gal, 1, out32.data_ptr())
        if rc:
            raise RuntimeError(L.tp_last_error(ctx._h).decode())

    for _ in range(args.warmup):
        step32()
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        step32()
    e1.record(st)
    torch.cuda.synchronize()
    t32 = e0.elapsed_time(e1) * 1e-3
    v32 = out32.cpu().numpy()
    r32 = np.abs(v32 - gpu_vals) / np.abs(gpu_vals)
    res["fp32_transforms"] = {"value": args.steps / t32, "unit": "fields/s", "ms_per_step": t32 / args.steps * 1e3,
                              "max_rel_vs_fp64": float(r32.max()), "median_rel_vs_fp64": float(np.median(r32)),
                              "outputs": int(r32.size)}
    plan32.close()
    # FP64 transforms: 5 F^2 log2(F^2) flop each, 3 + 2 per aperture per field
    F = int(L.tp_apm_fft_size(plan._h))
    flops = (3 + 2 * len(thetas)) * 5.0 * F * F * math.log2(F * F)
    f64_peak = tp.pipe_peaks(local)[2] * 2
    res["roofline"] = {"bound": "fp64", "achieved": flops / (t_dev / args.steps) / 1e12, "peak": f64_peak / 1e12,
                       "unit": "TFLOP/s", "frac": flops / (t_dev / args.steps) / f64_peak, "traffic": None,
                       "kernel": "the field's FP64 2-D transforms (cuFFT, 88% of the device time) and this "
                                 "library's kernels around them",
                       "work": "5 F^2 log2(F^2) flop per F x F transform",
                       "peak_source": "tp_pipe_peaks FP64 FMA/s x 2, measured now"}
    if not args.no_cpu_baseline:
        from oracle import aperture_mass as A

        # one aperture of the same field on the host (numpy/scipy, as the
        # reference), the field time = gridding + 4 x that aperture's map
        t0 = time.perf_counter()
        grid, w = A.cic_grid(x, y, g, npix, fs)
        t_grid = time.perf_counter() - t0
        t0 = time.perf_counter()
        A.map_weighted(grid, w, A.q_grid(npix, fs, thetas[0]))
        t_map = time.perf_counter() - t0
        t_field = t_grid + len(thetas) * t_map
        res["cpu_baseline"] = {"value": 1.0 / t_field, "unit": "fields/s", "cores": 1, "kind": "port",
                               "sample": f"CIC gridding + 1 of the 4 aperture maps of the same field timed "
                                         f"({t_grid:.2f} s + {t_map:.2f} s), field = gridding + 4 maps; "
                                         f"numpy/scipy as the reference"}
    plan.close()
    ctx.close()
    return res


def run_surrogate(args):
    """The b_kappa surrogate network of config 4: FP64 line-of-sight targets
    for --sg-cosmo Latin-hypercube cosmologies x --sg-points triangles each
    (2^24 points by default), Adam on the tensor-core network, the relative
    error of b_kappa on --sg-holdout other cosmologies, the forward rate of the
    host API, and the roofline of the GEMM every layer runs (65536 x 256 x 256,
    BF16, against the measured cuBLAS BF16 peak)."""
    import torch

    import threepoint_gb300 as tp
    from threepoint_gb300 import surrogate as S

    rank, world, local = dist_env()
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    zs, ns = nz_config()
    nz = tp.rebin_n_of_z(zs, ns, 256, 3.0)
    cos = S.lhs_box(args.sg_cosmo + args.sg_holdout, seed=LHS_SEED + 4)
    ctx = tp.Context(local)
    t0 = time.perf_counter()
    x, y = S.generate(ctx, cos[:args.sg_cosmo], nz, args.sg_points, seed=1)
    t_gen = time.perf_counter() - t0
    xh, yh = S.generate(ctx, cos[args.sg_cosmo:], nz, args.sg_holdout_points, seed=2)
    ctx.close()
    sg = S.Surrogate(max_batch=args.sg_batch, device=local, seed=0)
    t0 = time.perf_counter()
    hist = sg.fit(x, y, steps=args.sg_steps, batch=args.sg_batch, lr=args.sg_lr, lr_end=args.sg_lr * 1e-2,
                  log_every=max(1, args.sg_steps // 10))
    t_train = time.perf_counter() - t0
    held = sg.evaluate(xh, yh)
    train_sample = sg.evaluate(x[:65536], y[:65536])
    t0 = time.perf_counter()
    sg.net.forward(xh)
    t_fwd = time.perf_counter() - t0

    # GEMM roofline: CUDA events on the network's stream around each launch
    Mg, Ng, Kg = 65536, 256, 256
    g = torch.Generator().manual_seed(0)
    A = torch.randn(Mg, Kg, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(Ng, Kg, generator=g).to(torch.bfloat16).cuda()
    Cm = torch.empty(Mg, Ng, dtype=torch.float32, device="cuda")
    st = torch.cuda.ExternalStream(sg.net.stream_handle, device=local)
    for _ in range(3):
        sg.net.gemm_device(A, B, Cm)
    times = []
    for _ in range(20):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sg.net.gemm_device(A, B, Cm)
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    t_gemm = statistics.median(times)
    tflops = 2.0 * Mg * Ng * Kg / t_gemm / 1e12
    peak, src = 1900.0, "fallback 1.9 PFLOP/s"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst)"
    except Exception:
        pass
    sg.close()
    return {"metric": "b_kappa surrogate (config 4): held-out relative error of b_kappa, forward points/s",
            "value": len(yh) / t_fwd, "unit": "points/s", "n_gpus": 1, "steps": args.sg_steps, "warmup": 0,
            "ms_per_step": t_train / max(1, args.sg_steps) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"{args.sg_cosmo} LHS cosmologies x {args.sg_points} triangles (l1, l2 "
                                   f"log-uniform on [10, 4e4], l3 in range), FP64 line-of-sight targets; "
                                   f"{args.sg_holdout} held-out cosmologies x {args.sg_holdout_points}",
                       "network": "8-256-256-256-256-1 SiLU, BF16 operands, FP32 accumulation and master weights",
                       "optimizer": f"Adam, batch {args.sg_batch}, lr {args.sg_lr:g} -> {args.sg_lr * 1e-2:g}",
                       "value_timing": "host API tp_mlp_forward over the held-out points (copies included)"},
            "accuracy": {"held_out": held, "train_sample": train_sample},
            "training": {"points": int(len(y)), "generation_s": t_gen, "train_s": t_train, "loss_history": hist},
            "roofline": {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                         "traffic": None, "kernel": f"k_gemm_tc {Mg} x {Ng} x {Kg}", "peak_source": src,
                         "ms_per_launch": t_gemm * 1e3}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cosmo-per-step", type=int, default=64)
    ap.add_argument("--lmax", default="ref")
    ap.add_argument("--cpu-sample", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--region-cap", type=int, default=32768)
    ap.add_argument("--map3-cluster", type=int, default=1, choices=[0, 1, 2],
                    help="8-CTA clusters per integral: 0 never, 1 for batches smaller than the CTA slots, 2 always")
    ap.add_argument("--dump-costs", default="")
    ap.add_argument("--no-order", action="store_true")
    ap.add_argument("--no-fp64-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-pipeline", action="store_true", help="one context, steps run one after another")
    ap.add_argument("--apm-npix", type=int, default=4096, help="pixels per side of the aperture-mass grid")
    ap.add_argument("--workload", default="map3",
                    choices=["map3", "gamma", "cov", "halo", "surrogate", "plain", "apm"],
                    help="map3: the headline metric; gamma / cov / halo: the shear-3PCF grid and covariance "
                         "configurations (halo: the halo-model terms T5-T7); surrogate: training and accuracy of "
                         "the b_kappa network; plain: the FP64 form on the fiducial 20 triplets; apm: the FFT "
                         "aperture-mass measurement")
    ap.add_argument("--gamma-triangles", type=int, default=0, help="first N triangles of the grid (0 = all 1000)")
    ap.add_argument("--gamma-fp64-sample", type=int, default=20)
    ap.add_argument("--gamma-region-cap", type=int, default=32768,
                    help="regions per Gamma integral (the grid's small triangles need more than the default)")
    ap.add_argument("--cov-pairs", type=int, default=24)
    ap.add_argument("--cov-fp64-pairs", type=int, default=4)
    ap.add_argument("--cov-terms", default="T1,T2,T4", help="comma-separated subset of T1,T2,T4 (T5-T7: --workload halo)")
    ap.add_argument("--cov-fp64-terms", default="T2,T4",
                    help="terms also run in FP64 for the error (the square T1 at the cap takes minutes in FP64)")
    ap.add_argument("--cov-region-cap", type=int, default=0, help="regions per covariance integral (0: library default)")
    ap.add_argument("--halo-pairs", type=int, default=32)
    ap.add_argument("--halo-terms", default="T5,T7", help="comma-separated subset of T5,T6,T7")
    ap.add_argument("--halo-fp64-pairs", type=int, default=2)
    ap.add_argument("--halo-fp64-terms", default="T7", help="terms also run in FP64 (one FP64 T5 integral ~1 min)")
    ap.add_argument("--halo-cpu-terms", default="T7", help="terms the CPU oracle samples (one integral each)")
    ap.add_argument("--sg-cosmo", type=int, default=64)
    ap.add_argument("--sg-points", type=int, default=1 << 18, help="training triangles per cosmology")
    ap.add_argument("--sg-holdout", type=int, default=8)
    ap.add_argument("--sg-holdout-points", type=int, default=1 << 14)
    ap.add_argument("--sg-steps", type=int, default=20000)
    ap.add_argument("--sg-batch", type=int, default=65536)
    ap.add_argument("--sg-lr", type=float, default=2e-3)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        res = run_reference(args)
    elif args.workload == "gamma":
        res = run_gamma(args)
    elif args.workload == "cov":
        res = run_cov(args)
    elif args.workload == "halo":
        res = run_halo(args)
    elif args.workload == "surrogate":
        res = run_surrogate(args)
    elif args.workload == "plain":
        res = run_plain(args)
    elif args.workload == "apm":
        res = run_apm(args)
    else:
        res = run_ours(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
