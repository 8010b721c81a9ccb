"""Host-side logic of the b_kappa surrogate: feature scaling, the box test,
the triangle sampler and the Latin hypercube (no GPU)."""
import math

import numpy as np

from threepoint_gb300 import surrogate as S


def test_features_span_the_box():
    lo = [v[1] for v in S.BOX]
    hi = [v[2] for v in S.BOX]
    ell = np.array([[S.L_RANGE[0]] * 3, [S.L_RANGE[1]] * 3])
    f = S.features(ell, np.array([lo, hi]))
    assert np.allclose(f[0], -1.0) and np.allclose(f[1], 1.0)
    mid = S.features([[math.sqrt(S.L_RANGE[0] * S.L_RANGE[1])] * 3], np.add(lo, hi) / 2)
    assert np.allclose(mid, 0.0, atol=1e-12)


def test_in_box_and_sampler():
    rng = np.random.default_rng(0)
    ell = S.sample_triangles(rng, 5000)
    assert ell.shape == (5000, 3)
    assert np.all((ell >= S.L_RANGE[0]) & (ell <= S.L_RANGE[1]))
    # l3 closes the triangle for some phi
    assert np.all(ell[:, 2] <= ell[:, 0] + ell[:, 1] + 1e-9)
    assert np.all(ell[:, 2] >= np.abs(ell[:, 0] - ell[:, 1]) - 1e-9)
    cos = np.array([0.3, 0.8, 0.7, -1.0, 0.96])
    assert S.in_box(ell, cos).all()
    assert not S.in_box([[5.0, 100.0, 100.0]], cos)[0]
    assert not S.in_box([[100.0, 100.0, 100.0]], [0.5, 0.8, 0.7, -1.0, 0.96])[0]
    assert not S.in_box([[0.0, 100.0, 100.0]], cos)[0]


def test_lhs_box_strata():
    cs = S.lhs_box(64, seed=3)
    arr = S.cosmo_array(cs)
    for j, (_, lo, hi) in enumerate(S.BOX):
        u = (arr[:, j] - lo) / (hi - lo)
        assert np.array_equal(np.sort(np.floor(u * 64).astype(int)), np.arange(64))
    assert all(abs(c["om"] - c["omb"] - c["omc"]) < 1e-15 and abs(c["ow"] + c["om"] - 1) < 1e-15 for c in cs)
