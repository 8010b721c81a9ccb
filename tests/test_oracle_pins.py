"""The oracle against the reference's own host code (golden vectors generated by
tests/golden/make_golden.py from the reference's bispectrum.cu / hcubature.cpp)."""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import COSMO1

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_host.json")))


def test_nz_restatement_matches_fixture(nz256):
    assert np.array_equal(np.array(GOLD["nz256"]), nz256)


def test_tables_match_reference(oracle_tables):
    a = oracle_tables.arrays()
    for n in ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur"):
        ref = np.array(GOLD["tables"][n])
        rel = np.abs(a[n] - ref) / np.maximum(np.abs(ref), 1e-300)
        # f_K/g differ from the reference only through the 15-digit Gauss table
        assert rel.max() < 1e-12, (n, rel.max())
    assert a["norm"] == GOLD["norm"]


def test_scalar_functions_match_reference(oracle_tables):
    T = oracle_tables
    for k, v in GOLD["linear_pk"]:
        assert T.linear_pk(k) == pytest.approx(v, rel=1e-14)
    for r, j, v in GOLD["sigmam"]:
        assert T.sigmam(r, j) == pytest.approx(v, rel=1e-14)
    for z, v in GOLD["lgr"]:
        assert T.lgr(z) == pytest.approx(v, rel=1e-14)
    for k, z, v in GOLD["P_k_nonlinear"]:
        assert T.P_k_nonlinear(k, z) == pytest.approx(v, rel=1e-12)


def test_limber_integrand_matches_reference_off_first_node(oracle_tables):
    for ell, z, v in GOLD["limber_nodes"]:
        assert oracle_tables.limber_integrand(ell, z) == pytest.approx(v, rel=1e-11, abs=1e-300)


def test_first_node_clamp_is_deliberate(oracle_tables):
    """The two lowest Gauss nodes (z ~ 4.7e-4, 2.5e-3) lie below half a table
    bin, where the reference interpolates with table index -1 (an out-of-bounds
    read, bispectrum.cu:356-359); the oracle clamps to bin 0, i.e. uses the
    bin-0 values with total weight 1."""
    a, _ = O.gq96()
    low = [1.5 - 1.5 * x for x in a if (1.5 - 1.5 * x) / 3.0 * 256 < 0.5]
    assert len(low) == 2
    z0 = low[0]
    arr = oracle_tables.arrays()
    # with the clamp, the interpolated f_K at z0 is exactly bin 0's value
    didx = z0 / 3.0 * 256
    assert int(didx) == 0 and didx - int(didx) < 0.5
    # integrand_bkappa at z0 with ell's away from the cut-offs is finite
    v = oracle_tables.integrand_bkappa(z0, 100.0, 120.0, 150.0)
    assert np.isfinite(v)


def test_map3_with_reference_cubature(oracle_tables):
    for rec in GOLD["map3_ref_cubature"]:
        th = [x * O.ARCMIN for x in rec["theta_arcmin"]]
        v, e, n = oracle_tables.map3(th)
        assert v == pytest.approx(rec["value"], rel=1e-13)


@pytest.mark.skipif(O.ref_lib() is None, reason="reference harness not built here")
def test_oracle_cubature_bit_identical_to_reference():
    L, R = O.lib(), O.ref_lib()

    @O.INTEGRAND_V
    def f(ndim, npts, x, fdata, fdim, fval):
        for i in range(npts):
            a, b = x[i * ndim], x[i * ndim + 1]
            c = x[i * ndim + 2] if ndim > 2 else 0.0
            fval[i * fdim] = math.exp(-50 * ((a - 0.3) ** 2 + (b - 0.6) ** 2 + (c - 0.2) ** 2)) + 0.1 * a * b
            if fdim > 1:
                fval[i * fdim + 1] = math.sin(3 * a) * b
        return 0

    for dim, fdim in ((2, 1), (3, 1), (3, 2)):
        xmin, xmax = np.zeros(dim), np.ones(dim)
        res = []
        for fn in (L.orc_hcubature_v, R.ref_hcubature_v):
            v, e = np.zeros(fdim), np.zeros(fdim)
            fn(fdim, C.cast(f, C.c_void_p), None, dim, O._dp(xmin), O._dp(xmax), 0, 0, 1e-5, 3, O._dp(v), O._dp(e))
            res.append((v.copy(), e.copy()))
        assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


def test_oracle_cubature_1d_gauss_kronrod():
    L = O.lib()

    @O.INTEGRAND_V
    def f(ndim, npts, x, fdata, fdim, fval):
        for i in range(npts):
            fval[i] = math.exp(-x[i])
        return 0

    v, e = np.zeros(1), np.zeros(1)
    L.orc_hcubature_v(1, C.cast(f, C.c_void_p), None, 1, O._dp(np.array([0.0])), O._dp(np.array([3.0])), 0, 0,
                      1e-10, 3, O._dp(v), O._dp(e))
    assert v[0] == pytest.approx(1 - math.exp(-3), rel=1e-12)


def test_ogata_nodes_against_scipy_zeros():
    sp = pytest.importorskip("scipy.special")
    W = O.ogata_weights()
    h = 0.1
    for row, nu in ((0, 6), (2, 2)):
        zeros = sp.jn_zeros(nu, 32)
        xi = zeros / math.pi
        psi = np.pi * (h * xi) * np.tanh(np.pi / 2 * np.sinh(h * xi)) / h
        assert np.allclose(W[row, 1:], psi, rtol=1e-12)
        Jn1 = sp.jv(nu + 1, zeros)
        w = 2 / (np.pi * zeros * Jn1 ** 2)
        t = h * xi
        psip = (np.sinh(np.pi * np.sinh(t)) + np.pi * t * np.cosh(t)) / (np.cosh(np.pi * np.sinh(t)) + 1)
        prod = w * psi ** 3 * sp.jv(nu, psi) * psip
        # psi_k approaches the zeros of J_nu as k grows, so J_nu(psi_k) and the
        # product weights fall towards zero and are conditioned in absolute terms
        assert np.allclose(W[row + 1, 1:], prod, rtol=1e-10, atol=1e-10 * np.abs(prod).max())


def test_gamma0_known_answer_analytic_bispectrum(nz256):
    """Known answer for the Gamma integrand chain (Ogata nodes, A, alpha,
    betabar, phases, centroid rotation): with the analytic test bispectrum of
    classed_version/bispectrum.cpp:989-996 and the Ogata settings of the
    reference's test (h = 0.01, k up to 3.5: classed testGamma_analytical_bispectrum.cpp:94),
    Gamma^0 equals the closed form ggg (classed gamma.cpp:567-586) in modulus
    for every triangle, and equals -ggg for equilateral ones (the closed form's
    sign and projection convention). Triangles from 8' up, where k <= 3.5
    resolves the bispectrum's highest-ell components."""
    import ctypes as C

    from conftest import COSMO1

    T = O.Tables(COSMO1, nz256)
    T.set_analytic(True)
    L = O.lib()
    L.orc_set_ogata.argtypes = [C.c_double, C.c_int]
    arc = 2.9088820866e-4
    try:
        L.orc_set_ogata(0.01, 350)
        for tri in [(30, 30, 30), (8, 6, 3), (12, 10, 4), (50, 40, 20)]:
            x = [t * arc for t in tri]
            g, _ = T.gamma(0, *x, 1e-3)
            ga = O.ggg_analytic(*x)
            assert abs(abs(g) / abs(ga) - 1) < 1e-3, (tri, g, ga)
            if tri[0] == tri[1] == tri[2]:
                assert abs(g / ga + 1) < 1e-3, (tri, g, ga)
    finally:
        L.orc_set_ogata(0.1, 33)
    # the default (CUDA) Ogata rule is back
    w = O.ogata_weights()
    assert w.shape == (4, 33)


WN_CASES = [((4, 4, 4), (8, 8, 8)), ((4, 4, 8), (4, 8, 8))]


@pytest.mark.parametrize("a,b", WN_CASES)
def test_white_noise_covariance_brute_force(nz256, a, b):
    """Known answer for the covariance formulas (including the permutation
    tables of T1_total and T2_total): a Gaussian white-noise field on a pixel
    grid, whose estimator covariance is summed in real space
    (oracle/white_noise.py, after classed testCalculateCovarianceGaussianWhiteNoise.cpp),
    against the oracle's square-window T1_total and T2_total with the equivalent
    constant P(ell) = sigma^2 A_pix (sigma_eps^2 = 2 sigma^2, n = 1/A_pix).
    Tolerances: T1 is a 6-D cubature at relative tolerance 1e-2; the pixel
    grid (0.25' for 4'-8' apertures) adds ~1e-3."""
    from conftest import COSMO1
    from oracle import white_noise as WN

    arc = 2.9088820866e-4
    side, pix, sigma = 40 * arc, 0.25 * arc, 0.3
    th123, th456 = np.array(a) * arc, np.array(b) * arc
    t1, t2 = WN.t1_t2(th123, th456, side, pix, sigma)
    T = O.Tables(COSMO1, nz256)
    T.set_noise(np.sqrt(2) * sigma, 1 / pix ** 2, True)
    p = O.CovParams(1, side, side * side, 0.0)
    assert T.cov_total(1, p, th123, th456) == pytest.approx(t1, rel=1e-2)
    assert T.cov_total(2, p, th123, th456) == pytest.approx(t2, rel=2e-3)


# ---- halo model (cuda_version/halomodel.cu), T5 / T6 / T7 ------------------
def test_halo_tables_match_reference(oracle_tables):
    """sigma^2(m) and dsigma^2/dm tables of setSigma2 / setdSigma2dm: the
    oracle's restatement on its own cubature equals the reference's host code."""
    s2, ds2 = oracle_tables.halo_tables()
    assert np.array_equal(s2, np.array(GOLD["halo_tables"]["sig2"]))
    assert np.array_equal(ds2, np.array(GOLD["halo_tables"]["dsig2"]))


def test_halo_functions_match_reference(oracle_tables):
    T = oracle_tables
    for m, z, v in GOLD["hmf"]:
        assert T.hmf(m, z) == pytest.approx(v, rel=1e-13)
    for m, z, s2, ds2 in GOLD["get_sigma2"]:
        assert T.get_sigma2(m, z) == pytest.approx(s2, rel=1e-14)
        assert T.get_dsigma2(m, z) == pytest.approx(ds2, rel=1e-14)
    for k, m, z, v in GOLD["u_NFW"]:
        assert T.u_nfw(k, m, z) == pytest.approx(v, rel=1e-14, abs=1e-300)
    for m, z, c, r in GOLD["concentration"]:
        assert O.lib().orc_concentration(m, z) == c
        assert T.r_200(m) == r
    for x, si, ci in GOLD["SiCi"]:
        assert O.sici(x) == (si, ci)


def test_halo_cubature_bit_identical_to_reference(oracle_tables):
    """The reference's own hcubature_v on the oracle's T5 / T6 / T7 integrands
    (6-D and 7-D, loose tolerances) gives the oracle's value bit for bit."""
    T = oracle_tables
    deg = 0.017453
    for g in GOLD["halo_ref_cubature"]:
        T.set_noise(g["sigma"], g["n_arcmin2"] / O.ARCMIN ** 2, False)
        par = O.CovParams(g["geometry"], g["thetaMax_deg"] * deg, g["area_deg2"] * deg * deg, 0.0,
                          g.get("thetaMaxSmaller_deg", 0.0) * deg)
        th6 = [x * O.ARCMIN for x in g["theta_arcmin"]]
        h = O.lib().orc_halo_ctx_create(T._h, C.byref(par), g["term"], O._dp(np.array(th6)))
        lmax = O.lib().orc_halo_ctx_lmax(h)
        nlog = 4 if g["term"] == 7 else 3
        ndim = 6 if g["term"] == 5 else 7
        xmin = np.array([math.log(1e-4)] * nlog + [0.0] * (ndim - 1 - nlog) + [1e9])
        xmax = np.array([math.log(lmax)] * nlog + [2 * math.pi] * (ndim - 1 - nlog) + [1e17])
        v, e = np.zeros(1), np.zeros(1)
        fp = C.cast(O.lib().orc_integrand_halo_v, C.c_void_p).value
        O.lib().orc_hcubature_v(1, C.c_void_p(fp), h, ndim, O._dp(xmin), O._dp(xmax), 0, 0, g["rel"], 3, O._dp(v),
                                O._dp(e))
        O.lib().orc_halo_ctx_destroy(h)
        assert v[0] == g["raw_value"] and e[0] == g["raw_err"], g["term"]
    T.set_noise(0.0, 1.0, False)  # the fixture's default


def test_halo_total_terms_follow_reference_branches():
    """T5_total tests th0 == th1 twice, so (a, a, b) is integrated as (a, a, a);
    T6_total's case E and T7_total's single ordering."""
    a, b, c = 1.0, 2.0, 3.0
    assert O.halo_total_terms(5, [a, a, b], [c, c, c]) == [(9, (0, 0, 0, 3, 3, 3))]
    assert sum(m for m, _ in O.halo_total_terms(5, [a, b, c], [a, b, c])) == 9
    assert O.halo_total_terms(6, [a, a, b], [c, c, c]) == [(1, (0, 0, 2, 3, 3, 3)), (2, (0, 2, 0, 3, 3, 3)),
                                                          (3, (3, 3, 0, 0, 2, 3))]
    assert O.halo_total_terms(7, [a, b, c], [c, b, a]) == [(1, (0, 1, 2, 3, 4, 5))]
