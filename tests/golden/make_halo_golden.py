"""Golden vectors of the reference's OWN halo-model device code
(trispectrum_limber_integrated / pentaspectrum_limber_integrated,
cuda_version/halomodel.cu:392-510), run on a GB300.

Three steps, as for make_device_golden.py:

1. ``prepare <reference cuda_version dir>`` (where the reference tree
   exists): builds the reference's z-tables and its sigma^2(m) /
   dsigma^2/dm mass tables with its own host code (oracle/_ref/libref_host.so)
   and compiles its device code with the harness kernels
   (oracle/_ref/ref_device.cubin); writes the inputs to
   oracle/_ref/halo_inputs.npz.
2. ``run [out.npz]`` (on the GPU machine; numpy and the CUDA driver only):
   uploads the constants copyConstants / set_cosmology / initHalomodel upload
   (bispectrum.cu:90-219, halomodel.cu:18-29), runs ref_halo_los and writes
   the outputs (default gpurun_out/ref_halo_out.npz).
3. ``finish [out.npz]``: merges inputs and outputs into
   tests/golden/reference_halo.npz, the committed fixture the tests read.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, HERE)

import make_device_golden as MD  # noqa: E402

INPUTS = os.path.join(MD.REF_DIR, "halo_inputs.npz")
FIXTURE = os.path.join(HERE, "reference_halo.npz")
NM = 128


def points(n=64, seed=5):
    """(m, l1, ..., l6): m log-uniform in [1e9, 1e17] Msun/h, ell log-uniform
    in [1e-3, 1e4] (the range the T5-T7 integrals reach)."""
    rng = np.random.default_rng(seed)
    m = 10 ** rng.uniform(9.0, 17.0, n)
    ell = 10 ** rng.uniform(-3.0, 4.0, (n, 6))
    return np.column_stack([m, ell])


def prepare(ref_tree):
    import subprocess

    import oracle as O
    from conftest import nz_table

    for target in ("ref", "refdev"):
        r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), target, "REF=" + ref_tree],
                           capture_output=True, text=True)
        if r.returncode:
            raise SystemExit(r.stdout + r.stderr)
    R = O.ref_lib()
    zs, ns = nz_table()
    nz = O.read_n_of_z(zs, ns, MD.NZB, 3.0)
    a96, w96 = np.zeros(48), np.zeros(48)
    R.ref_gq96(O._dp(a96), O._dp(w96))
    cos = MD.cosmologies()[:3]  # fiducial and two box corners
    tabs, halo, cvec = [], [], []
    for c in cos:
        R.ref_set_cosmo(*[c[k] for k in MD.COSMO_KEYS])
        out = np.zeros(6 * MD.NZB + 1)
        R.ref_build_tables(O._dp(nz), O._dp(out))
        ht = np.zeros(2 * NM)
        R.ref_halo_tables(O._dp(ht))
        tabs.append(out)
        halo.append(ht)
        cvec.append([c[k] for k in MD.COSMO_KEYS])
    np.savez(INPUTS, cosmo=np.array(cvec), tables=np.array(tabs), halo=np.array(halo), a96=a96, w96=w96,
             pk_given=np.zeros(len(cos), dtype=np.int32), pk=np.zeros(MD.NZB), pk_grid=np.zeros(3),
             ogata=O.ogata_weights(), pts=points())
    print("wrote", INPUTS, "and", MD.CUBIN)


def run(out_path):
    inp = dict(np.load(INPUTS))
    D = MD.Driver()
    pts = inp["pts"]
    n = len(pts)
    d_p, d_t, d_q = D.alloc(pts.nbytes, pts), D.alloc(8 * n), D.alloc(8 * n)
    tri, pen = [], []
    for ci in range(len(inp["cosmo"])):
        MD.upload_cosmology(D, inp, ci)
        # initHalomodel (halomodel.cu:18-29)
        D.set("devLogMmin", 9.0)
        D.set("devLogMmax", 17.0)
        D.set("dev_n_mbins", NM, np.int32)
        D.set("dev_sigma2_array", inp["halo"][ci][:NM])
        D.set("dev_dSigma2dm_array", inp["halo"][ci][NM:])
        D.launch("ref_halo_los", (n + 31) // 32, 32, [d_p, MD.C.c_int(n), d_t, d_q])
        tri.append(D.get(d_t, n))
        pen.append(D.get(d_q, n))
    for p in (d_p, d_t, d_q):
        D.free(p)
    res = {"tri": np.array(tri), "penta": np.array(pen)}
    os.makedirs(os.path.dirname(os.path.abspath(out_path)), exist_ok=True)
    np.savez(out_path, **res)
    print("wrote", out_path, {k: v.shape for k, v in res.items()},
          "finite:", all(np.isfinite(v).all() for v in res.values()))


def finish(out_path):
    inp = dict(np.load(INPUTS))
    res = dict(np.load(out_path))
    np.savez_compressed(FIXTURE, cosmo=inp["cosmo"], halo=inp["halo"], pts=inp["pts"], **res)
    print("wrote", FIXTURE, os.path.getsize(FIXTURE), "bytes")


if __name__ == "__main__":
    if len(sys.argv) < 2 or sys.argv[1] not in ("prepare", "run", "finish"):
        raise SystemExit("usage: make_halo_golden.py prepare <reference cuda_version dir> | run [out.npz] | "
                         "finish [out.npz]")
    step = sys.argv[1]
    if step == "prepare":
        if len(sys.argv) < 3:
            raise SystemExit("prepare needs the reference's cuda_version directory")
        prepare(sys.argv[2])
    else:
        path = sys.argv[2] if len(sys.argv) > 2 else os.path.join(ROOT, "gpurun_out", "ref_halo_out.npz")
        run(path) if step == "run" else finish(path)
