"""Generate the golden vectors that pin the oracle to the reference's own code.

Run in a checkout where the reference tree is available and
``make -C oracle ref`` has built ``oracle/_ref/libref_host.so`` (the reference's
cuda_version/bispectrum.cu host functions and vendored hcubature.cpp behind a
thin C harness). Writes ``tests/golden/reference_host.json``. The fixture is
committed; the tests read it on machines without the reference tree.
"""
import ctypes as C
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import oracle as O  # noqa: E402
from conftest import COSMO1, nz_table  # noqa: E402


def main():
    R = O.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libref_host.so missing: run `make -C oracle ref` where the reference exists")
    zs, ns = nz_table()
    nz = O.read_n_of_z(zs, ns, 256, 3.0)
    c = COSMO1
    R.ref_set_cosmo(*[c[k] for k in ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")])
    out = np.zeros(6 * 256 + 1)
    R.ref_build_tables(O._dp(nz), O._dp(out))
    g = {"cosmology": c, "nz256": nz.tolist()}
    names = ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur")
    g["tables"] = {n: out[i * 256:(i + 1) * 256].tolist() for i, n in enumerate(names)}
    g["norm"] = out[-1]
    # scalar functions of the reference's host code
    g["linear_pk"] = [[k, R.ref_linear_pk(k)] for k in (1e-4, 1e-3, 1e-2, 0.1, 1.0, 10.0, 100.0)]
    g["sigmam"] = [[r, j, R.ref_sigmam(r, j)] for r, j in ((8.0, 0), (1.0, 1), (0.5, 2), (0.5, 3))]
    g["lgr"] = [[z, R.ref_lgr(z)] for z in (0.0, 0.5, 1.0, 3.0)]
    g["P_k_nonlinear"] = [[k, z, R.ref_P_k_nonlinear(k, z)] for k, z in ((0.1, 0.5), (1.0, 1.0), (10.0, 2.0))]
    # P_kappa LOS integrand at the 96 nodes of [0, z_max] except those below half
    # a bin (z/z_max*255 < 0.5), where the reference interpolates with table
    # index -1 (bispectrum.cu:389-392)
    a, w = O.gq96()
    nodes = sorted([1.5 - 1.5 * x for x in a] + [1.5 + 1.5 * x for x in a])
    g["limber_nodes"] = [[ell, z, R.ref_limber_integrand(ell, z)] for ell in (100.0, 3000.0) for z in nodes
                         if z / 3.0 * 255 >= 0.5]
    # the reference's hcubature_v on the oracle's <Map^3> integrand
    T = O.Tables(c, nz)
    L = O.lib()
    fptr = C.cast(L.orc_integrand_map3_v, C.c_void_p).value
    g["map3_ref_cubature"] = []
    for th in ((16, 16, 16), (8, 16, 16)):
        t = [x * O.ARCMIN for x in th]
        ctx = L.orc_map3_ctx_create(T._h, *t)
        lmax = 10 / min(t)
        xmin = np.array([1.0, 1.0, 0.0])
        xmax = np.array([lmax, lmax, 2 * math.pi])
        v, e = np.zeros(1), np.zeros(1)
        R.ref_hcubature_v(1, C.c_void_p(fptr), ctx, 3, O._dp(xmin), O._dp(xmax), 0, 0, 1e-4, 3, O._dp(v), O._dp(e))
        L.orc_map3_ctx_destroy(ctx)
        g["map3_ref_cubature"].append({"theta_arcmin": th, "value": v[0] / (2 * math.pi) ** 3,
                                       "err": e[0] / (2 * math.pi) ** 3})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_host.json")
    with open(path, "w") as f:
        json.dump(g, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main()
