"""bench.py pieces that need no GPU: the module imports, every workload
parses, and the reference-work figure reads roofline.json."""
import importlib.util
import json
import os
import subprocess
import sys

from conftest import ROOT


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def test_reference_work_reads_roofline_json():
    b = load_bench()
    with open(os.path.join(ROOT, "roofline.json")) as f:
        per_point = json.load(f)["map3_point"]["flop_equivalent"]
    r = b.reference_work(2.0e9, 1.2)
    assert r["flop_equivalent_per_point"] == per_point
    assert abs(r["tflop_equivalent_per_s"] - 2.0e9 * per_point / 1.2 / 1e12) < 1e-9


def test_every_workload_parses():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         cwd=ROOT, timeout=120)
    assert out.returncode == 0
    for w in ("map3", "gamma", "cov", "surrogate", "plain"):
        assert w in out.stdout


def test_workload_helpers():
    b = load_bench()
    assert len(b.thetas_220()) == 220
    cs = b.lhs_cosmologies(16, seed=1)
    assert len(cs) == 16 and all(abs(c["om"] - c["omb"] - c["omc"]) < 1e-15 for c in cs)


def test_output_errors_and_corners():
    import numpy as np

    bench = load_bench()
    v64 = np.array([1.0, 2.0, 0.0, -4.0])
    v32 = np.array([1.0005, 2.0, 0.0, -4.0])
    r = bench.output_errors(v32, v64)
    assert r["outputs"] == 4 and r["nonzero_outputs"] == 3 and r["zero_valued_agree"]
    assert abs(r["max_rel"] - 5e-4) < 1e-12 and r["outputs_above_1e-3"] == 0
    assert not bench.output_errors(np.array([1e-30, 1.0]), np.array([0.0, 1.0]))["zero_valued_agree"]
    cs = bench.corner_cosmologies()
    assert len(cs) == 4
    for key, lo, hi in (("om", 0.2, 0.4), ("sigma8", 0.7, 0.9), ("h", 0.6, 0.8), ("w", -1.2, -0.8), ("ns", 0.92, 1.0)):
        assert {c[key] for c in cs} == {lo, hi}, key
