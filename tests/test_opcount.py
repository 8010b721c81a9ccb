"""The operation-counting restatement of the reference's per-point formula
(oracle/opcount.py) against the oracle's values, and roofline.json against a
fresh count."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import COSMO1, ROOT
from oracle import opcount as OC


@pytest.fixture(scope="module")
def model(oracle_tables):
    a, w = np.zeros(48), np.zeros(48)
    O.lib().orc_gq96(O._dp(a), O._dp(w))
    return OC.Model(COSMO1, oracle_tables.arrays(), a, w)


def test_restatement_reproduces_the_oracle(model, oracle_tables):
    for k1, k2, k3, z in [(0.1, 0.2, 0.25, 0.5), (1.0, 1.5, 2.0, 1.2), (5.0, 5.0, 5.0, 0.05), (0.02, 3.0, 3.01, 2.9)]:
        zn = OC.N(z)
        didx = zn / model.z_max * 256
        idx = int(didx.v)
        v, _ = OC.count(model.bispec, OC.N(k1), OC.N(k2), OC.N(k3), zn, idx, didx - idx)
        assert v == pytest.approx(oracle_tables.bispec_at_z(k1, k2, k3, z), rel=1e-13)
    ell = (300.0, 500.0, 600.0)
    assert OC.count(model.bkappa, *map(OC.N, ell))[0] == pytest.approx(oracle_tables.bkappa(*ell), rel=1e-13)
    th = np.array([2.0, 4.0, 8.0]) * O.ARCMIN
    l1, l2, phi = 400.0, 900.0, 2.0
    l3 = math.sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * math.cos(phi))
    u = O.lib().orc_uHat
    ref = l1 * l2 * oracle_tables.bkappa(l1, l2, l3) * u(l1 * th[0]) * u(l2 * th[1]) * u(l3 * th[2])
    assert OC.count(model.map3_point, l1, l2, phi, th)[0] == pytest.approx(ref, rel=1e-13)


def test_roofline_json_is_current():
    import importlib.util

    spec = importlib.util.spec_from_file_location("mk", os.path.join(ROOT, "oracle", "make_roofline_json.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    fresh = mk.build()
    with open(os.path.join(ROOT, "roofline.json")) as f:
        committed = json.load(f)
    assert committed["weights"] == fresh["weights"]
    for k in ("bispec", "map3_point"):
        assert committed[k]["flop_equivalent"] == pytest.approx(fresh[k]["flop_equivalent"], rel=1e-12)
