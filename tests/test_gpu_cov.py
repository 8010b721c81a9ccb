"""P(ell) and the <Map^3> covariance terms T1, T2, T4 on the GPU against the oracle."""
import numpy as np
import pytest

import oracle as O
from conftest import COSMO1

pytestmark = pytest.mark.gpu
ARC = O.ARCMIN
DEG = 0.017453
SIG, NGAL = 0.3, 10 / ARC ** 2  # sigma_eps, n_gal = 10 arcmin^-2 in rad^-2
TMAX, AREA = 10 * DEG, 100 * DEG * DEG
TH6 = [8 * ARC, 8 * ARC, 16 * ARC, 8 * ARC, 16 * ARC, 16 * ARC]


@pytest.fixture(scope="module")
def cov_ctx(nz256):
    import threepoint_gb300 as tp

    ctx = tp.Context(0)
    ctx.set_shape_noise(SIG, NGAL, False)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def cov_oracle(nz256):
    T = O.Tables(COSMO1, nz256)
    T.set_noise(SIG, NGAL, False)
    O.set_threads(0)
    return T


def params(geom, lmin=0.0):
    return O.CovParams(geom, TMAX, AREA, lmin)


def test_pell_matches_oracle(cov_ctx, cov_oracle):
    ell = np.exp(np.linspace(np.log(1.0), np.log(1e5), 40))
    got = cov_ctx.Pell(ell, precision=0)
    ref = np.array([cov_oracle.Pell(l) for l in ell])
    assert np.max(np.abs(got - ref) / ref) < 1e-11
    got32 = cov_ctx.Pell(ell, precision=1)
    assert np.max(np.abs(got32 - ref) / ref) < 1e-4


def test_t1_infinite_matches_oracle(cov_ctx, cov_oracle):
    got = cov_ctx.cov_term(1, TH6, geometry=2, thetaMax=TMAX, area=AREA, precision=0)[0]
    ref = cov_oracle.cov_T(1, params(2), TH6)[0]
    assert got == pytest.approx(ref, rel=1e-6)
    got32 = cov_ctx.cov_term(1, TH6, geometry=2, thetaMax=TMAX, area=AREA, precision=1)[0]
    assert got32 == pytest.approx(ref, rel=1e-3)


def test_t2_square_matches_oracle(cov_ctx, cov_oracle):
    got = cov_ctx.cov_term(2, TH6, geometry=1, thetaMax=TMAX, area=AREA, precision=0)[0]
    ref = cov_oracle.cov_T(2, params(1), TH6)[0]
    assert got == pytest.approx(ref, rel=1e-6)


def test_t4_matches_oracle(cov_ctx, cov_oracle):
    got = cov_ctx.cov_term(4, TH6, geometry=2, thetaMax=TMAX, area=AREA, precision=0)[0]
    ref = cov_oracle.cov_T(4, params(2), TH6)[0]
    assert got == pytest.approx(ref, rel=1e-6)
    got32 = cov_ctx.cov_term(4, TH6, geometry=2, thetaMax=TMAX, area=AREA, precision=1)[0]
    assert got32 == pytest.approx(ref, rel=1e-3)


@pytest.fixture(scope="module")
def shapenoise_ctx(nz256):
    import threepoint_gb300 as tp

    ctx = tp.Context(0)
    ctx.set_shape_noise(SIG, NGAL, True)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def shapenoise_oracle(nz256):
    T = O.Tables(COSMO1, nz256)
    T.set_noise(SIG, NGAL, True)
    return T


def test_t1_square_shapenoise_matches_oracle(shapenoise_ctx, shapenoise_oracle):
    got = shapenoise_ctx.cov_term(1, TH6, geometry=1, thetaMax=TMAX, area=AREA, precision=0)[0]
    ref = shapenoise_oracle.cov_T(1, params(1), TH6)[0]
    assert got == pytest.approx(ref, rel=1e-6)


@pytest.mark.parametrize("term", [1, 2])
def test_rectangle_matches_oracle(shapenoise_ctx, shapenoise_oracle, term):
    """Rectangular survey (G_rectangle, sides thetaMax and thetaMax_smaller)."""
    import threepoint_gb300 as tp

    small = 0.4 * TMAX
    shapenoise_ctx.set_rectangle_side(small)
    got = shapenoise_ctx.cov_term(term, TH6, geometry=tp.GEOM_RECTANGLE, thetaMax=TMAX, area=AREA, precision=0)[0]
    ref = shapenoise_oracle.cov_T(term, O.CovParams(3, TMAX, AREA, 0.0, small), TH6)[0]
    assert got == pytest.approx(ref, rel=1e-5 if term == 1 else 1e-6)
    # a rectangle with equal sides is the square
    shapenoise_ctx.set_rectangle_side(TMAX)
    sq = shapenoise_ctx.cov_term(term, TH6, geometry=tp.GEOM_SQUARE, thetaMax=TMAX, area=AREA, precision=0)[0]
    re = shapenoise_ctx.cov_term(term, TH6, geometry=tp.GEOM_RECTANGLE, thetaMax=TMAX, area=AREA, precision=0)[0]
    assert re == sq


def test_t4_only_infinite(cov_ctx):
    """The reference's T4 throws for finite geometries; here TP_ERR_ARG."""
    import threepoint_gb300 as tp

    for geom in (tp.GEOM_CIRCLE, tp.GEOM_SQUARE, tp.GEOM_RECTANGLE):
        with pytest.raises(tp.ThreepointError):
            cov_ctx.cov_term(4, TH6, geometry=geom, thetaMax=TMAX, area=AREA)


@pytest.mark.parametrize("term,geom", [(1, 2), (2, 1), (1, 1)])
def test_totals_match_oracle(shapenoise_ctx, shapenoise_oracle, term, geom):
    """The permutation tables of T1_total/T2_total against the oracle's, over
    every equality pattern of the two triplets (shape-noise-only P)."""
    a_s = [(4, 4, 4), (4, 4, 8), (4, 8, 8), (4, 8, 4), (2, 4, 8)]
    b_s = [(8, 8, 8), (8, 8, 16), (8, 16, 8), (8, 16, 16), (4, 8, 16)]
    if term == 1 and geom == 1:
        a_s, b_s = a_s[:2], b_s[:3]
    pairs = [(np.array(a) * ARC, np.array(b) * ARC) for a in a_s for b in b_s]
    A = np.array([p[0] for p in pairs])
    B = np.array([p[1] for p in pairs])
    got = shapenoise_ctx.cov_total(term, A, B, geometry=geom, thetaMax=TMAX, area=AREA, precision=0)
    ref = np.array([shapenoise_oracle.cov_total(term, params(geom), a, b) for a, b in pairs])
    # the 6-D square-window T1 runs at the reference's relative tolerance 1e-2,
    # where last-bit differences of the integrand can move a few region splits
    rtol = 1e-5 if (term == 1 and geom == 1) else 1e-6
    assert np.allclose(got, ref, rtol=rtol, atol=0), np.abs(got / ref - 1).max()


def test_t4_total_permutation_table(cov_ctx):
    """T4_total reproduces the reference's argument patterns (including its
    uneven th4==th5 branch): checked against sums of single T4 terms."""
    a = np.array([4, 4, 8]) * ARC
    b = np.array([8, 16, 16]) * ARC
    # th0==th1 branch, else sub-branch: 6 terms
    t = [(1, (b[0], a[0], a[0], a[2], b[1], b[2])), (2, (b[0], a[0], a[2], a[0], b[1], b[2])),
         (1, (b[1], a[0], a[0], a[2], b[0], b[2])), (2, (b[1], a[0], a[2], a[0], b[0], b[2])),
         (1, (b[2], a[0], a[0], a[2], b[0], b[1])), (2, (b[2], a[0], a[2], a[0], b[0], b[1]))]
    singles = cov_ctx.cov_term(4, [x[1] for x in t], geometry=2, thetaMax=TMAX, area=AREA, precision=1)
    total = cov_ctx.cov_total(4, [a], [b], geometry=2, thetaMax=TMAX, area=AREA, precision=1)[0]
    assert total == pytest.approx(sum(m * s for (m, _), s in zip(t, singles)), rel=1e-12)


def test_t1_total_symmetry(shapenoise_ctx):
    """Covariance symmetry under swapping the two triplets (infinite field)."""
    a = np.array([4, 4, 8]) * ARC
    b = np.array([8, 8, 16]) * ARC
    ab = shapenoise_ctx.cov_total(1, [a], [b], geometry=2, thetaMax=TMAX, area=AREA)[0]
    ba = shapenoise_ctx.cov_total(1, [b], [a], geometry=2, thetaMax=TMAX, area=AREA)[0]
    assert ab == pytest.approx(ba, rel=1e-3)


@pytest.mark.parametrize("a,b", [((4, 4, 4), (8, 8, 8)), ((4, 4, 8), (4, 8, 8))])
def test_white_noise_brute_force_on_gpu(nz256, a, b):
    """The GPU T1_total/T2_total (square window, constant P) against the
    real-space white-noise brute force of oracle/white_noise.py."""
    import threepoint_gb300 as tp
    from oracle import white_noise as WN

    side, pix, sigma = 40 * ARC, 0.25 * ARC, 0.3
    th123, th456 = np.array(a) * ARC, np.array(b) * ARC
    t1, t2 = WN.t1_t2(th123, th456, side, pix, sigma)
    ctx = tp.Context(0)
    ctx.set_shape_noise(np.sqrt(2) * sigma, 1 / pix ** 2, True)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    kw = dict(geometry=tp.GEOM_SQUARE, thetaMax=side, area=side * side, precision=tp.FP64)
    assert ctx.cov_total(1, [th123], [th456], **kw)[0] == pytest.approx(t1, rel=1e-2)
    assert ctx.cov_total(2, [th123], [th456], **kw)[0] == pytest.approx(t2, rel=2e-3)
    ctx.close()
