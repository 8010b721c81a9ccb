"""Pins against the reference's OWN device code.

tests/golden/reference_device.npz holds bispec, integrand_bkappa and the
Gamma integrands as the reference's cuda_version/bispectrum.cu and gamma.cu
compute them on a GB300 (harness oracle/ref_device.cu, script
tests/golden/make_device_golden.py), from tables its own host code built, for
the fiducial cosmology, the four corners of the Latin-hypercube box and the
fiducial cosmology with a given linear P(k) table. The oracle (CPU) and the
GPU path (FP64 and FP32) are compared with those values.
"""
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import nz_table

GOLD_PATH = os.path.join(os.path.dirname(__file__), "golden", "reference_device.npz")
pytestmark = pytest.mark.skipif(not os.path.exists(GOLD_PATH), reason="reference device fixture not generated")
KEYS = ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")
NZB = 256
H0_OVER_C = 100.0 / 299792.0


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD_PATH))


@pytest.fixture(scope="module")
def nz():
    zs, ns = nz_table()
    return O.read_n_of_z(zs, ns, NZB, 3.0)


def cosmo(g, ci):
    return dict(zip(KEYS, g["cosmo"][ci]))


def pk_args(g, ci):
    if not g["pk_given"][ci]:
        return {}
    dk, kmin, kmax = g["pk_grid"]
    return dict(pk=g["pk"], dk=float(dk), kmin=float(kmin), kmax=float(kmax))


def interp_mid(tab, z, zmax):
    """The reference's mid-bin two-point interpolation (bispectrum.cu:335-437)
    for z in [dz/2, z_max)."""
    f = z / zmax * NZB
    i = int(f)
    d = f - i
    w = 1 - abs(d - 0.5)
    j = i
    if d > 0.5:
        j = i if i == NZB - 1 else i + 1
        if i == NZB - 1:
            return tab[i] * w
    elif d < 0.5:
        j = i - 1
    return tab[i] * w + tab[j] * (1 - w)


def node_weights(g):
    """Gauss weight x dx of each of the 96 line-of-sight nodes (exact nodes,
    the GPU path's and the oracle's)."""
    a, w = O.gq96()
    wq = np.empty(96)
    wq[0::2] = w * 1.5
    wq[1::2] = w * 1.5
    return wq


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


# ---------------------------------------------------------------------------
# the oracle against the reference's device code (CPU)
def test_oracle_bispec_and_integrand_match_reference_device(gold, nz):
    ell, z = gold["ell"], gold["node_z"][gold["node_safe"]]
    worst_b, worst_i = [], []
    for ci in range(len(gold["cosmo"])):
        c = cosmo(gold, ci)
        T = O.Tables(c, nz, **pk_args(gold, ci))
        fk_tab = gold["tables"][ci][:NZB]
        rb, ri = [], []
        for a, (l1, l2, l3) in enumerate(ell):
            for b, zz in enumerate(z):
                fk = interp_mid(fk_tab, zz, c["zmax"])
                rb.append(rel(T.bispec_at_z(l1 / fk, l2 / fk, l3 / fk, zz), gold["bispec"][ci, a, b]))
                ri.append(rel(T.integrand_bkappa(zz, l1, l2, l3), gold["integrand"][ci, a, b]))
        worst_b.append((np.median(rb), np.max(rb)))
        worst_i.append((np.median(ri), np.max(ri)))
    mb = max(x[1] for x in worst_b)
    mi = max(x[1] for x in worst_i)
    assert max(x[0] for x in worst_b) < 1e-13 and mb < 1e-10, worst_b
    assert max(x[0] for x in worst_i) < 1e-13 and mi < 1e-10, worst_i


def test_oracle_gamma_integrand_matches_reference_device(gold, nz):
    pts = gold["gamma_pts"]
    for a, ci in enumerate(gold["gamma_cosmo"]):
        T = O.Tables(cosmo(gold, int(ci)), nz, **pk_args(gold, int(ci)))
        for b, x in enumerate(gold["gamma_tri"]):
            for which in (0, 1):
                got = T.gamma_integrand_points(which, *x, pts)
                ref = gold["gamma"][a, b, which]
                scale = np.max(np.abs(ref))
                assert np.max(np.abs(got - ref)) < 1e-11 * scale, (ci, b, which)


def test_reference_device_fixture_is_finite_and_nonzero(gold):
    for k in ("bispec", "integrand", "gamma"):
        assert np.isfinite(gold[k]).all(), k
        assert np.count_nonzero(gold[k]) > 0.9 * gold[k].size, k


# ---------------------------------------------------------------------------
# the GPU path against the reference's device code
@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_bkappa_nodes_match_reference_device(gold, nz, precision):
    from conftest import gpu_available

    if not gpu_available():
        pytest.skip("no CUDA device")
    import threepoint_gb300 as tp

    safe = gold["node_safe"]
    wq = node_weights(gold)[safe]
    out = []
    with tp.Context(0) as ctx:
        for ci in range(len(gold["cosmo"])):
            c = cosmo(gold, ci)
            ctx.set_cosmology(tp.cosmology(**c), nz, **pk_args(gold, ci))
            term, bis = ctx.bkappa_nodes(gold["ell"], 0, precision=precision)
            pref = 27.0 / 8.0 * c["om"] ** 3 * H0_OVER_C ** 5
            ref_term = gold["integrand"][ci] * wq[None, :] * pref
            ref_b = gold["bispec"][ci]
            got_b, got_t = bis[:, safe], term[:, safe]
            # g(z) vanishes at the last nodes before z_max: there the reference's
            # integrand is exactly 0 and ours must be negligible
            zero = ref_term == 0
            assert np.all(np.abs(got_t[zero]) <= 1e-12 * np.abs(ref_term).max()), ci
            # median of the per-node relative error, and the largest error
            # relative to the triangle's largest node value (the 3-halo F2 + d_n q
            # factor can cancel at single nodes of squeezed triangles)
            sb = np.abs(ref_b).max(1, keepdims=True)
            st = np.abs(ref_term).max(1, keepdims=True)
            out.append((ci, np.median(rel(got_b, ref_b)), np.max(np.abs(got_b - ref_b) / sb),
                        np.median(rel(got_t[~zero], ref_term[~zero])), np.max(np.abs(got_t - ref_term) / st)))
    # FP64: last-bit differences of the exp2/log2 form against the
    # reference's pow(10, .) grow with the squeezed triangles' ell ratios (up to
    # 3e4 here) through F2_tree: 6e-11 of the triangle's largest node value,
    # 4e-9 for the most squeezed one. FP32 (approximate ex2/rcp): the 3-halo sum
    # of F2-weighted P_i P_j products cancels at single nodes of squeezed
    # triangles, so a node's B can be off by ~1e-3 of the triangle's largest
    # one; the line-of-sight terms, which the integrals sum, stay within 1e-3.
    tol_med, tol_b, tol_t = (1e-12, 1e-8, 1e-8) if precision == 0 else (3e-5, 1e-2, 1e-3)
    for ci, mb, xb, mt, xt in out:
        assert mb < tol_med and xb < tol_b, ("bispec", out)
        assert mt < tol_med and xt < tol_t, ("term", out)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_gpu_gamma_integrand_matches_reference_device(gold, nz, precision):
    from conftest import gpu_available

    if not gpu_available():
        pytest.skip("no CUDA device")
    import threepoint_gb300 as tp

    pts = gold["gamma_pts"]
    tol = 1e-10 if precision == 0 else 1e-3
    with tp.Context(0) as ctx:
        for a, ci in enumerate(gold["gamma_cosmo"]):
            ctx.set_cosmology(tp.cosmology(**cosmo(gold, int(ci))), nz, **pk_args(gold, int(ci)))
            for b, x in enumerate(gold["gamma_tri"]):
                for which in (0, 1):
                    got = ctx.gamma_integrand_points(which, x, pts, precision=precision)
                    ref = gold["gamma"][a, b, which]
                    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
                    assert err < tol, (int(ci), b, which, err)


HALO_PATH = os.path.join(os.path.dirname(__file__), "golden", "reference_halo.npz")


@pytest.mark.skipif(not os.path.exists(HALO_PATH), reason="reference halo fixture not generated")
def test_oracle_halo_los_matches_reference_device_code(nz):
    """trispectrum_limber_integrated / pentaspectrum_limber_integrated as the
    reference's halomodel.cu computes them on a GB300 (harness kernel
    ref_halo_los, script tests/golden/make_halo_golden.py) with the mass tables
    its host code built, against the oracle's restatement; the fixture's mass
    tables equal the oracle's bit for bit."""
    f = np.load(HALO_PATH)
    for ci in range(len(f["cosmo"])):
        T = O.Tables(dict(zip(KEYS, f["cosmo"][ci])), nz)
        s2, ds2 = T.halo_tables()
        assert np.array_equal(s2, f["halo"][ci][:128]) and np.array_equal(ds2, f["halo"][ci][128:])
        tri, pen = T.halo_los(f["pts"])
        np.testing.assert_allclose(tri, f["tri"][ci], rtol=1e-10, atol=0)
        np.testing.assert_allclose(pen, f["penta"][ci], rtol=1e-10, atol=0)
