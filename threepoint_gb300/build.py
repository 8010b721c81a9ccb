"""Build recipe of libthreepoint_gb300.so (sm_103a only).

Every translation unit is compiled by nvcc in parallel and linked in-tree into
``threepoint_gb300/build/libthreepoint_gb300.so``. No CMake, no
torch.utils.cpp_extension: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libthreepoint_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]


CLI = os.path.join(HERE, "cli")
BIN = os.path.join(BUILD, "bin")
# command-line drivers, named like the reference's executables
CLIS = ("calculateApertureStatistics", "calculateGamma", "calculateApertureStatisticsCovariance")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], capture_output=True, check=True)
            return c
        except Exception:
            continue
    raise RuntimeError("nvcc not found")


def _deps_mtime():
    m = 0.0
    for d in (CSRC, CLI, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    t = os.path.join(HERE, "tuned.json")
    return max(m, os.path.getmtime(t)) if os.path.exists(t) else m


def _cli_cmds():
    cxx = os.environ.get("CXX", "g++")
    return [[cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), os.path.join(CLI, c + ".cpp"),
             "-L" + BUILD, "-lthreepoint_gb300", "-Wl,-rpath,$ORIGIN/..", "-o", os.path.join(BIN, c + ".x")]
            for c in CLIS]


def tuned_flags():
    """-D flags of the kernel launch shape chosen by the autotuner (tuned.json)"""
    try:
        with open(os.path.join(HERE, "tuned.json")) as f:
            cfg = json.load(f).get("k_map3", {})
    except (OSError, ValueError):
        return []
    return [f"-D{k}={int(v)}" for k, v in sorted(cfg.items()) if k.startswith("TP_MAP3_")]


def build(force: bool = False, verbose: bool = False, extra=(), use_tuned: bool = True) -> str:
    os.makedirs(BIN, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime() and all(
            os.path.exists(os.path.join(BIN, c + ".x")) for c in CLIS):
        return LIB
    nvcc = _nvcc()
    if use_tuned:
        given = {e.split("=")[0] for e in extra if e.startswith("-D")}
        extra = [f for f in tuned_flags() if f.split("=")[0] not in given] + list(extra)
    objs = []
    cmds = []
    for s in sources():
        o = os.path.join(BUILD, os.path.splitext(s)[0] + ".o")
        objs.append(o)
        cmds.append([nvcc, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, s), "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed on " + cmd[-3])
    link = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    with cf.ThreadPoolExecutor(max_workers=len(CLIS)) as ex:
        for cmd, r in ex.map(run, _cli_cmds()):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("driver build failed: " + cmd[-1])
    return LIB


def driver(name: str) -> str:
    """Path of a built command-line driver (calculateGamma etc.)."""
    return os.path.join(BIN, name + ".x")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
