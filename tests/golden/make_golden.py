"""Generate the golden vectors that pin the oracle to the reference's own code.

Run in a checkout where the reference tree is available and
``make -C oracle ref`` has built ``oracle/_ref/libref_host.so`` (the reference's
cuda_version/bispectrum.cu host functions and vendored hcubature.cpp behind a
thin C harness; its halo-model host functions from cuda_version/halomodel.cu
too). Writes ``tests/golden/reference_host.json``. The fixture is
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
    # halo model (cuda_version/halomodel.cu): the sigma^2(m) tables of
    # setSigma2 / setdSigma2dm and host evaluations of its __host__ __device__
    # functions after the tables are filled
    ht = np.zeros(256)
    R.ref_halo_tables(O._dp(ht))
    g["halo_tables"] = {"sig2": ht[:128].tolist(), "dsig2": ht[128:].tolist()}
    rng = np.random.default_rng(11)
    ms, zz = 10 ** rng.uniform(9, 17, 24), rng.uniform(0.02, 2.98, 24)
    ks = 10 ** rng.uniform(-3, 3, 24)
    g["hmf"] = [[m, z, R.ref_hmf(m, z)] for m, z in zip(ms, zz)]
    g["get_sigma2"] = [[m, z, R.ref_get_sigma2(m, z), R.ref_get_dSigma2dm(m, z)] for m, z in zip(ms, zz)]
    g["u_NFW"] = [[k, m, z, R.ref_u_NFW(k, m, z)] for k, m, z in zip(ks, ms, zz)]
    g["concentration"] = [[m, z, R.ref_concentration(m, z), R.ref_r_200(m, z)] for m, z in zip(ms, zz)]
    sici = []
    for x in np.concatenate([10 ** rng.uniform(-3, 4, 24), [3.999, 4.0, 4.001]]):
        si, ci = C.c_double(), C.c_double()
        R.ref_SiCi(float(x), C.byref(si), C.byref(ci))
        sici.append([float(x), si.value, ci.value])
    g["SiCi"] = sici
    # the reference's hcubature_v on the oracle's T5 / T6 / T7 integrands at
    # loose tolerances (the reference's own 1e-2 / 1e-1 take 1e6 and more points)
    T.set_noise(0.3, 10 / O.ARCMIN ** 2, False)
    deg = 0.017453
    g["halo_ref_cubature"] = []
    for term, geom, rel in ((5, 2, 0.2), (6, 1, 0.5), (6, 3, 0.5), (7, 2, 0.3)):
        th6 = [x * O.ARCMIN for x in (8, 8, 16, 8, 16, 16)]
        par = O.CovParams(geom, 10 * deg, 100 * deg * deg, 0.0, 5 * deg)
        h = L.orc_halo_ctx_create(T._h, C.byref(par), term, O._dp(np.array(th6)))
        lmax = L.orc_halo_ctx_lmax(h)
        ll, lh = math.log(1e-4), math.log(lmax)
        nlog = 4 if term == 7 else 3
        ndim = 6 if term == 5 else 7
        xmin = np.array([ll] * nlog + [0.0] * (ndim - 1 - nlog) + [1e9])
        xmax = np.array([lh] * nlog + [2 * math.pi] * (ndim - 1 - nlog) + [1e17])
        v, e = np.zeros(1), np.zeros(1)
        fp = C.cast(L.orc_integrand_halo_v, C.c_void_p).value
        R.ref_hcubature_v(1, C.c_void_p(fp), h, ndim, O._dp(xmin), O._dp(xmax), 0, 0, rel, 3, O._dp(v), O._dp(e))
        L.orc_halo_ctx_destroy(h)
        g["halo_ref_cubature"].append({"term": term, "geometry": geom, "rel": rel, "theta_arcmin": [8, 8, 16, 8, 16, 16],
                                       "thetaMax_deg": 10, "thetaMaxSmaller_deg": 5, "area_deg2": 100,
                                       "sigma": 0.3, "n_arcmin2": 10,
                                       "raw_value": v[0], "raw_err": e[0]})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_host.json")
    with open(path, "w") as f:
        json.dump(g, f, indent=0)
    print("wrote", path)


if __name__ == "__main__":
    main()
