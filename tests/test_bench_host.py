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
    assert abs(r["achieved_tflop_equivalent_per_s"] - 2.0e9 * per_point / 1.2 / 1e12) < 1e-9


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
