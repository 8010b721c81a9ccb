"""Writes roofline.json: the reference's operation counts per bispec call, per
96-node b_kappa and per <Map^3> cubature point, counted by oracle/opcount.py
(a restatement checked against the oracle) at seeded sample points of the
fiducial cosmology, with the FLOP weights of the convention.

    python oracle/make_roofline_json.py            # writes <repo>/roofline.json
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from oracle import opcount as OC  # noqa: E402

COSMO = dict(h=0.7, sigma8=0.8, omb=0.048, ns=0.96, w=-1.0, om=0.3, zmax=3.0, ow=0.7, omc=0.252)
ARCMIN = 2.9088820866e-4


def model():
    zs = np.arange(3001) * 1e-3
    ns = zs ** 2 * np.exp(-(zs / 0.5) ** 1.5)
    T = O.Tables(COSMO, O.read_n_of_z(zs, ns, 256, 3.0))
    a, w = np.zeros(48), np.zeros(48)
    O.lib().orc_gq96(O._dp(a), O._dp(w))
    return T, OC.Model(COSMO, T.arrays(), a, w)


def mean_counts(samples):
    tot = {}
    for c in samples:
        for k, v in c.items():
            tot[k] = tot.get(k, 0) + v
    return {k: v / len(samples) for k, v in sorted(tot.items())}


def build():
    T, M = model()
    rng = np.random.default_rng(20261203)
    bis, pts = [], []
    for _ in range(8):
        k = np.exp(rng.uniform(math.log(0.01), math.log(10.0), 3))
        z = float(rng.uniform(0.05, 2.9))
        zn = OC.N(z)
        didx = zn / M.z_max * 256
        idx = int(didx.v)
        bis.append(OC.count(M.bispec, *[OC.N(x) for x in k], zn, idx, didx - idx)[1])
    th = np.array([2.0, 4.0, 8.0]) * ARCMIN
    for _ in range(4):
        l1, l2 = np.exp(rng.uniform(math.log(10.0), math.log(5000.0), 2))
        phi = float(rng.uniform(0.0, 2 * math.pi))
        pts.append(OC.count(M.map3_point, float(l1), float(l2), phi, th)[1])
    cb, cp = mean_counts(bis), mean_counts(pts)
    return {
        "what": "operations of the reference's FP64 formula chain (cuda_version/bispectrum.cu, "
                "apertureStatistics.cu:138-153), counted by oracle/opcount.py",
        "weights": OC.WEIGHTS,
        "bispec": {"counts": cb, "flop_equivalent": OC.flop_equivalent(cb), "samples": len(bis)},
        "map3_point": {"counts": cp, "flop_equivalent": OC.flop_equivalent(cp), "samples": len(pts),
                       "note": "one cubature point: l3, one 96-node b_kappa (96 integrand_bkappa, each one "
                               "bispec), three uHat"},
        "per_integral": "N_eval (evaluated cubature points, 33 per region in 3-D) x map3_point.flop_equivalent",
    }


if __name__ == "__main__":
    doc = build()
    with open(os.path.join(ROOT, "roofline.json"), "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps({k: doc[k]["flop_equivalent"] for k in ("bispec", "map3_point")}))
