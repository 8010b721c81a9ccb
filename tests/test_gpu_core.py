"""GPU parity of the table build, b_kappa and <Map^3> against the CPU oracle."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import COSMO1

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_host.json")))
ARC = O.ARCMIN


def test_tables_match_oracle(gpu_ctx, oracle_tables):
    g = gpu_ctx.tables(0)
    o = oracle_tables.arrays()
    for n in ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur"):
        rel = np.abs(g[n] - o[n]) / np.maximum(np.abs(o[n]), 1e-300)
        assert rel.max() < 1e-10, (n, rel.max())
    assert g["norm"] == pytest.approx(o["norm"], rel=1e-12)


def test_tables_match_reference_golden(gpu_ctx):
    g = gpu_ctx.tables(0)
    for n in ("D1", "r_sigma", "n_eff", "ncur"):
        ref = np.array(GOLD["tables"][n])
        assert np.max(np.abs(g[n] - ref) / np.abs(ref)) < 1e-10, n


def random_triangles(n, seed=0, lmin=1.0, lmax=1e5):
    rng = np.random.default_rng(seed)
    l1 = np.exp(rng.uniform(np.log(lmin), np.log(lmax), n))
    l2 = np.exp(rng.uniform(np.log(lmin), np.log(lmax), n))
    phi = rng.uniform(0, 2 * np.pi, n)
    l3 = np.sqrt(l1 ** 2 + l2 ** 2 + 2 * l1 * l2 * np.cos(phi))
    return np.stack([l1, l2, l3], 1)


def test_bkappa_fp64_matches_oracle(gpu_ctx, oracle_tables):
    ell = random_triangles(512, seed=1)
    got = gpu_ctx.bkappa(ell, precision=0)
    ref = oracle_tables.bkappa_batch(ell)
    rel = np.abs(got - ref) / np.abs(ref)
    # the tree-level kernel F2 is scale-free but ill-conditioned for squeezed
    # triangles (ell ratios up to 1e5 here): last-bit differences of the inputs
    # grow by up to that ratio
    assert np.median(rel) < 1e-13 and rel.max() < 1e-8, (np.median(rel), rel.max())


def test_bkappa_fp32_within_tolerance(gpu_ctx, oracle_tables):
    ell = random_triangles(512, seed=2)
    got = gpu_ctx.bkappa(ell, precision=1)
    ref = oracle_tables.bkappa_batch(ell)
    rel = np.abs(got - ref) / np.abs(ref)
    assert np.median(rel) < 1e-5 and rel.max() < 1e-3, (np.median(rel), rel.max())


def test_bkappa_edge_cases(gpu_ctx):
    ell = np.array([[0.0, 10.0, 10.0], [10.0, 10.0, 0.0], [1e-11, 5.0, 5.0], [100.0, 100.0, 100.0]])
    got = gpu_ctx.bkappa(ell, precision=0)
    assert got[0] == 0 and got[1] == 0 and got[2] == 0 and got[3] > 0


def test_map3_fp64_matches_reference_cubature_golden(gpu_ctx):
    for rec in GOLD["map3_ref_cubature"]:
        th = [x * ARC for x in rec["theta_arcmin"]]
        v = gpu_ctx.MapMapMap(th, precision=0)
        assert v == pytest.approx(rec["value"], rel=1e-6), (rec["theta_arcmin"], v, rec["value"])


def test_map3_fp64_matches_oracle(gpu_ctx, oracle_tables):
    O.set_threads(os.cpu_count() or 8)
    for th_arc in ((4, 8, 16), (2, 2, 2)):
        th = [x * ARC for x in th_arc]
        ref, err, nev = oracle_tables.map3(th)
        got, info = gpu_ctx.map3_batch([th], precision=0, return_info=True)
        assert got[0, 0] == pytest.approx(ref, rel=1e-6), (th_arc, got[0, 0], ref)
        # same adaptive decisions: evaluation counts agree to a few regions
        assert abs(int(info["neval"][0, 0]) - nev) <= 0.01 * nev, (int(info["neval"][0, 0]), nev)


def test_map3_fp32_against_fp64(gpu_ctx):
    # includes strongly unequal triplets whose first-rule values are far below
    # the float range but non-zero in FP64
    trip = ((2, 4, 8), (16, 16, 16), (4, 4, 16), (1.4697, 3.1748, 21.772), (2.1544, 14.812, 32.0))
    th = [[a * ARC, b * ARC, c * ARC] for a, b, c in trip]
    v64 = gpu_ctx.map3_batch(th, precision=0)
    v32 = gpu_ctx.map3_batch(th, precision=1)
    assert np.all(v64 != 0)
    rel = np.abs(v32 - v64) / np.abs(v64)
    assert rel.max() < 1e-3, rel


def test_map3_fp32_against_fp64_wide_radii(gpu_ctx):
    """FP32 against FP64 over radii 0.5' to 100' (ell up to 7e4 at the
    smallest radius): the FP32 node evaluation (packed pairs, merged
    reciprocals with their out-of-range fallback) stays within 1e-3."""
    radii = (0.5, 2.0, 8.0, 32.0, 100.0)
    trip = [(a, b, c) for i, a in enumerate(radii) for j, b in enumerate(radii[i:], i)
            for c in radii[j:]][::2]
    th = [[a * ARC, b * ARC, c * ARC] for a, b, c in trip]
    v64 = gpu_ctx.map3_batch(th, precision=0)
    v32 = gpu_ctx.map3_batch(th, precision=1)
    assert np.array_equal(v32 == 0, v64 == 0)
    nz = v64 != 0
    rel = np.abs(v32[nz] - v64[nz]) / np.abs(v64[nz])
    assert rel.max() < 1e-3, (rel.max(), np.array(trip)[np.argmax(np.abs(v32 - v64)[0])])


def test_map3_zero_for_disjoint_filters(gpu_ctx, oracle_tables):
    # (1', 1.47', 32'): all 33 points of the first rule have a zero filter
    # product in FP64, so the reference's cubature stops at 0 after one region
    th = [1.0 * ARC, 1.4697 * ARC, 32.0 * ARC]
    assert oracle_tables.map3(th)[0] == 0.0
    for prec in (0, 1):
        v, info = gpu_ctx.map3_batch([th], precision=prec, return_info=True)
        assert v[0, 0] == 0.0 and info["neval"][0, 0] == 33


def test_map3_batch_over_cosmologies(nz256):
    import threepoint_gb300 as tp

    cos = [tp.cosmology(**COSMO1), tp.cosmology.flat(0.25, 0.75, 0.65, -0.9, 0.95)]
    with tp.Context(0) as ctx:
        ctx.set_cosmologies(cos, nz256)
        th = [[8 * ARC, 8 * ARC, 16 * ARC], [16 * ARC, 16 * ARC, 16 * ARC]]
        both = ctx.map3_batch(th, precision=0)
        one = ctx.map3_batch(th, cosmo_index=[1], precision=0)
        assert np.array_equal(both[1], one[0])
        T2 = O.Tables(dict(h=0.65, sigma8=0.75, omb=0.048, ns=0.95, w=-0.9, om=0.25, ow=0.75, omc=0.202,
                           zmax=3.0), nz256)
        ref = T2.map3(th[1])[0]
        assert both[1, 1] == pytest.approx(ref, rel=1e-6)


def test_invalid_arguments_raise(gpu_ctx):
    import threepoint_gb300 as tp

    with pytest.raises(tp.ThreepointError):
        gpu_ctx.map3_batch([[0.0, 1e-3, 1e-3]])
    with pytest.raises(tp.ThreepointError):
        gpu_ctx.map3_batch([[1e-3, 1e-3, 1e-3]], cosmo_index=[5])
    with pytest.raises(tp.ThreepointError):
        gpu_ctx.bkappa([[1.0, 1.0, 1.0]], cosmo_index=[3])


def test_region_cap_exhaustion_reports_and_recovers(nz256):
    """A forced region-cap exhaustion: the call reports TP_ERR_CAPACITY with
    the per-integral status and still writes the value; the context stays
    usable and the same integral converges once the cap allows it."""
    import threepoint_gb300 as tp

    arc = 2.9088820866e-4
    th = [[1 * arc, 1 * arc, 1 * arc]]
    ctx = tp.Context(0)
    with pytest.raises(tp.ThreepointError):
        ctx.set_limits(region_cap=63)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    ctx.set_limits(region_cap=64)
    ctx.set_escalation(0)  # report the cap instead of integrating again
    with pytest.raises(tp.ThreepointError) as e:
        ctx.map3_batch(th, precision=tp.FP32)
    assert e.value.status == tp.TP_ERR_CAPACITY
    v, info = ctx.map3_batch(th, precision=tp.FP32, return_info=True, check=False)
    assert info["status"][0, 0] & 1  # region cap
    assert np.isfinite(v).all()
    ctx.set_limits(region_cap=32768)
    v2, info2 = ctx.map3_batch(th, precision=tp.FP32, return_info=True)
    assert info2["status"][0, 0] == 0
    ref = ctx.map3_batch(th, precision=tp.FP64)
    assert v2[0, 0] == pytest.approx(ref[0, 0], rel=1e-3)
    ctx.close()


def test_bkappa_on_reference_dump_grid(gpu_ctx, oracle_tables):
    """b_kappa on the grid of the reference's bispectrum dump program
    (classed testApertureStatistics_bispectrum.cpp:59-65: 10 log-spaced ell on
    [1, 1e5] x 10 ell x 10 phi on [1e-4, 2 pi]), FP64 against the oracle, and
    the points the reference's own cut-offs set to zero (ell3 <= 1e-10)."""
    ls = np.logspace(0, 5, 10)
    phis = np.linspace(1e-4, 6.28308531, 10)
    ell = np.array([(a, b, math.sqrt(max(a * a + b * b + 2 * a * b * math.cos(p), 0.0)))
                    for a in ls for b in ls for p in phis])
    got = gpu_ctx.bkappa(ell, precision=0)
    ref = oracle_tables.bkappa_batch(ell)
    nz = ref != 0
    assert np.array_equal(got == 0, ref == 0)
    rel = np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])
    assert np.median(rel) < 1e-13 and rel.max() < 1e-8, (np.median(rel), rel.max())
    got32 = gpu_ctx.bkappa(ell, precision=1)
    rel32 = np.abs(got32[nz] - ref[nz]) / np.abs(ref[nz])
    assert np.median(rel32) < 1e-5 and rel32.max() < 1e-3, (np.median(rel32), rel32.max())


def test_bkappa_nodes_sum_to_bkappa_and_match_oracle(gpu_ctx, oracle_tables):
    """tp_bkappa_nodes: the 96 line-of-sight terms of a triangle sum to
    tp_bkappa_batch's b_kappa, and each term equals the oracle's
    integrand_bkappa at that node times the Gauss weight and prefactor."""
    ell = random_triangles(16, seed=5, lmin=10.0, lmax=4e4)
    a, w = O.gq96()
    z = np.empty(96)
    z[0::2], z[1::2] = 1.5 - 1.5 * a, 1.5 + 1.5 * a
    wq = np.repeat(w * 1.5, 2)
    pref = 27.0 / 8.0 * COSMO1["om"] ** 3 * (100.0 / 299792.0) ** 5
    for prec, tol_sum, tol_node in ((0, 1e-12, 1e-10), (1, 1e-5, 1e-3)):
        term, bis = gpu_ctx.bkappa_nodes(ell, 0, precision=prec)
        tot = gpu_ctx.bkappa(ell, precision=prec)
        assert np.max(np.abs(term.sum(1) - tot) / np.abs(tot)) < tol_sum
        ref = np.array([[oracle_tables.integrand_bkappa(zz, *e) * wq[j] * pref for j, zz in enumerate(z)]
                        for e in ell])
        # g(z) vanishes at the last nodes before z_max: those terms are exactly 0
        nzm = ref != 0
        assert np.all(np.abs(term[~nzm]) <= 1e-12 * np.abs(ref).max())
        r = np.abs(term[nzm] - ref[nzm]) / np.abs(ref[nzm])
        # largest error relative to the triangle's largest node term: single
        # nodes can sit where the 3-halo factor F2 + d_n q changes sign
        rs = np.abs(term - ref) / np.abs(ref).max(1, keepdims=True)
        assert np.median(r) < tol_node * 1e-2 and rs.max() < tol_node, (prec, np.median(r), rs.max())


def test_gamma_integrand_points_match_oracle(gpu_ctx, oracle_tables):
    rng = np.random.default_rng(11)
    pts = np.stack([rng.uniform(0.01, 2.99, 32), rng.uniform(0, 2 * np.pi, 32), rng.uniform(0.01, 1.56, 32)], 1)
    x = np.array([4.0, 6.0, 8.0]) * ARC
    for which in (0, 1):
        ref = oracle_tables.gamma_integrand_points(which, *x, pts)
        for prec, tol in ((0, 1e-10), (1, 1e-3)):
            got = gpu_ctx.gamma_integrand_points(which, x, pts, precision=prec)
            assert np.max(np.abs(got - ref)) < tol * np.max(np.abs(ref)), (which, prec)


def test_region_cap_escalation_reproduces_uncapped_result(nz256):
    """With escalation on (the default), an integral that reaches a small
    region cap is integrated again with larger caps; the value equals the one
    of a run with a cap large enough from the start, bit for bit, since the
    adaptive sequence is the same."""
    import threepoint_gb300 as tp

    th = [[1 * ARC, 1 * ARC, 1 * ARC], [16 * ARC, 16 * ARC, 16 * ARC]]
    with tp.Context(0) as ctx:
        ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
        ref, info_ref = ctx.map3_batch(th, precision=tp.FP32, return_info=True)
        ctx.set_limits(region_cap=64)
        got, info = ctx.map3_batch(th, precision=tp.FP32, return_info=True)
    assert np.all(info["status"] == 0)
    assert np.array_equal(got, ref) and np.array_equal(info["neval"], info_ref["neval"])


def test_map3_fp64_matches_oracle_at_box_corner(nz256):
    """FP64 <Map^3> at a corner of the Latin-hypercube box (Omega_m 0.4,
    sigma_8 0.9, h 0.8, w -0.8, n_s 1.0) on every 40th of the 220 triplets of
    10 log-spaced radii 1'-32', against the oracle, with the same number of
    cubature points (same adaptive decisions) within 1%."""
    import threepoint_gb300 as tp

    O.set_threads(os.cpu_count() or 8)
    c = dict(h=0.8, sigma8=0.9, omb=0.048, ns=1.0, w=-0.8, om=0.4, ow=0.6, omc=0.352, zmax=3.0)
    radii = np.exp(np.linspace(0.0, np.log(32.0), 10)) * ARC
    trip = [(radii[i], radii[j], radii[k]) for i in range(10) for j in range(i, 10) for k in range(j, 10)][::40]
    T = O.Tables(c, nz256)
    with tp.Context(0) as ctx:
        ctx.set_cosmology(tp.cosmology(**c), nz256)
        got, info = ctx.map3_batch(trip, precision=tp.FP64, return_info=True)
    for t, th in enumerate(trip):
        ref, err, nev = T.map3(list(th))
        if ref == 0:
            assert got[0, t] == 0
            continue
        assert got[0, t] == pytest.approx(ref, rel=1e-6), (np.array(th) / ARC, got[0, t], ref)
        assert abs(int(info["neval"][0, t]) - nev) <= 0.01 * nev


@pytest.mark.parametrize("prec", [0, 1])
def test_map3_cluster_equals_one_cta(gpu_ctx, prec):
    """A batch smaller than the device's CTA slots runs one 8-CTA cluster per
    integral; the same regions are refined as with one CTA, so values, error
    estimates and evaluation counts are identical."""
    r = np.array([2.0, 4.0, 8.0, 16.0]) * ARC
    th = np.array([(r[i], r[j], r[k]) for i in range(4) for j in range(i, 4) for k in range(j, 4)])
    try:
        gpu_ctx.set_map3_cluster(False)
        a, ia = gpu_ctx.map3_batch(th, cosmo_index=[0], precision=prec, return_info=True)
        gpu_ctx.set_map3_cluster(True)
        b, ib = gpu_ctx.map3_batch(th, cosmo_index=[0], precision=prec, return_info=True)
    finally:
        gpu_ctx.set_map3_cluster(True)
    assert np.array_equal(a, b)
    assert np.array_equal(ia["err"], ib["err"]) and np.array_equal(ia["neval"], ib["neval"])
    assert np.all(np.isfinite(a))
