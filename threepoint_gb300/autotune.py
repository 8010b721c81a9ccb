"""Autotuner of the <Map^3> kernel's launch shape.

The FP32 kernel k_map3<float> has four build-time knobs (tp_map3.cu):
TP_MAP3_MINB (CTAs per SM requested from the register allocator: 4 -> 64
registers per thread, 3 -> 80, 2 -> 128), TP_MAP3_UNROLL (node pairs per loop
iteration), TP_MAP3_DUP_IN_LOOP (triangle pairs held in registers or formed
at use) and TP_MAP3_PLT_GLOBAL (linear-P(k) table in shared memory or read
through L1; the latter is what lets four CTAs fit an SM). The tuner builds the library for every candidate, times the kernel on
a fixed batch (64 seeded cosmologies x 220 aperture-radius triplets, the
benchmark step's size, FP32,
device-resident, CUDA events, best of 3 launches after a warm-up), writes the
fastest to threepoint_gb300/tuned.json and rebuilds with it. build() passes
tuned.json's values as -D flags.

    python -m threepoint_gb300.autotune            # sweep, write tuned.json, rebuild
    python -m threepoint_gb300.autotune --measure  # time the current build (one JSON line)
"""
from __future__ import annotations

import itertools
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "tuned.json")
ARCMIN = 2.9088820866e-4
KNOBS = {"TP_MAP3_MINB": (3, 2), "TP_MAP3_UNROLL": (1, 2), "TP_MAP3_DUP_IN_LOOP": (1, 0), "TP_MAP3_PLT_GLOBAL": (0,)}


def _workload(n_cosmo=64, seed=20261203):
    rng = np.random.default_rng(seed)
    u = (rng.permutation(n_cosmo)[:, None] + rng.uniform(size=(n_cosmo, 5))) / n_cosmo
    lo = np.array([0.2, 0.7, 0.6, -1.2, 0.92])
    hi = np.array([0.4, 0.9, 0.8, -0.8, 1.0])
    p = lo + u * (hi - lo)
    cos = [dict(om=a, sigma8=b, h=c, w=d, ns=e) for a, b, c, d, e in p]
    radii = np.exp(np.linspace(0.0, np.log(32.0), 10)) * ARCMIN
    th = np.array([(radii[i], radii[j], radii[k]) for i in range(10) for j in range(i, 10) for k in range(j, 10)])
    zs = np.arange(3001) * 1e-3
    ns = zs ** 2 * np.exp(-(zs / 0.5) ** 1.5)
    return cos, th, zs, ns


def measure(device=0):
    """ms per k_map3<float> launch of the fixed batch with the current build"""
    import torch

    import threepoint_gb300 as tp

    torch.cuda.set_device(device)
    cos, th, zs, ns = _workload()
    ctx = tp.Context(device)
    ctx.set_cosmologies([tp.cosmology.flat(c["om"], c["sigma8"], c["h"], c["w"], c["ns"]) for c in cos],
                        tp.rebin_n_of_z(zs, ns, 256, 3.0))
    dev = torch.device("cuda", device)
    nc, nt = len(cos), len(th)
    jc = torch.arange(nc, dtype=torch.int32, device=dev).repeat_interleave(nt)
    jt = torch.tensor(np.tile(th, (nc, 1)), dtype=torch.float64, device=dev)
    out = torch.zeros(nc * nt, dtype=torch.float64, device=dev)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=device)
    best = float("inf")
    for rep in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            ctx.map3_jobs_device(jc, jt, out, precision=tp.FP32)
            e1.record(stream)
        torch.cuda.synchronize()
        if rep > 0:
            best = min(best, e0.elapsed_time(e1))
    ctx.close()
    return best


def sweep(device=0, knobs=None):
    from threepoint_gb300 import build as B

    results = []
    knobs = knobs or KNOBS
    for vals in itertools.product(*knobs.values()):
        cfg = dict(zip(knobs, vals))
        flags = [f"-D{k}={v}" for k, v in cfg.items()]
        B.build(force=True, extra=flags, use_tuned=False)
        r = subprocess.run([sys.executable, "-m", "threepoint_gb300.autotune", "--measure", "--device", str(device)],
                           capture_output=True, text=True, cwd=os.path.dirname(HERE))
        ms = json.loads(r.stdout.strip().splitlines()[-1])["ms"] if r.returncode == 0 else None
        results.append({"config": cfg, "ms": ms})
        print(json.dumps(results[-1]), flush=True)
    ok = [r for r in results if r["ms"] is not None]
    if not ok:
        raise RuntimeError("no candidate ran")
    best = min(ok, key=lambda r: r["ms"])
    import torch

    doc = {"k_map3": best["config"],
           "measured": {"device": torch.cuda.get_device_name(device), "date": time.strftime("%Y-%m-%d"),
                        "workload": "64 seeded LHS cosmologies x 220 triplets, FP32, best of 3 launches",
                        "candidates": results},
           "command": "python -m threepoint_gb300.autotune"}
    with open(TUNED, "w") as f:
        json.dump(doc, f, indent=1)
    B.build(force=True)
    return doc


def main():
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--measure", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--knobs", default="", help='JSON {"TP_MAP3_MINB": [3, 4], ...} replacing the default candidates')
    a = ap.parse_args()
    if a.measure:
        print(json.dumps({"ms": measure(a.device)}))
    else:
        doc = sweep(a.device, json.loads(a.knobs) if a.knobs else None)
        print(json.dumps({"best": doc["k_map3"]}))


if __name__ == "__main__":
    main()
