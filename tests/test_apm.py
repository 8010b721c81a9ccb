"""FFT aperture-mass measurement (python_scripts/aperture_mass_computer.py):
the numpy restatement against the reference module's own outputs
(tests/golden/reference_apm.npz, made by tests/golden/make_apm_golden.py), and
the GPU path against both."""
import os

import numpy as np
import pytest

from oracle import aperture_mass as A

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_apm.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_oracle_matches_reference_module(gold):
    x, y, g = gold["x"], gold["y"], gold["g"]
    n, fs, th = int(gold["npix"]), float(gold["fieldsize"]), list(gold["thetas"])
    grid, w = A.cic_grid(x, y, g, n, fs)
    assert rel(grid, gold["shears"]) < 1e-13 and rel(w, gold["norm"]) < 1e-13
    assert rel(A.map_weighted(grid, w, A.q_grid(n, fs, 2.0)), gold["map_theta2"]) < 1e-12
    assert rel(A.map_weighted(grid, w, A.q_grid(n, fs, 2.0, True)), gold["map_theta2_poly"]) < 1e-12
    for poly in (False, True):
        maps = np.array([A.map_weighted(grid, w, A.q_grid(n, fs, t, poly)) for t in th])
        for same in (False, True):
            got = A.map3_of_maps(maps, th, fs, same, poly)
            assert rel(got, gold[f"map3_poly{int(poly)}_same{int(same)}"]) < 1e-11, (poly, same)
    assert rel(A.extract_map3(x, y, g, n, th, fs), gold["map3_catalogue"]) < 1e-11


def test_oracle_cic_conserves_weight():
    rng = np.random.default_rng(1)
    x, y = rng.uniform(0, 30, 1000), rng.uniform(0, 30, 1000)
    g = rng.standard_normal(1000) + 1j * rng.standard_normal(1000)
    grid, w = A.cic_grid(x, y, g, 40, 30.0)
    # every galaxy lands with weights summing to 1 unless a corner leaves the
    # last bin edge (x + cell beyond 40/39 * 30 is impossible for x <= 30)
    assert abs(w.sum() - 1000) < 1e-9
    assert abs(grid.sum() - g.sum()) < 1e-9


def _gpu():
    from conftest import gpu_available

    if not gpu_available():
        pytest.skip("no CUDA device")
    import threepoint_gb300 as tp
    from threepoint_gb300 import aperture_mass as G

    return tp, G


@pytest.mark.gpu
def test_gpu_matches_reference_module(gold):
    tp, G = _gpu()
    x, y, g = gold["x"], gold["y"], gold["g"]
    n, fs, th = int(gold["npix"]), float(gold["fieldsize"]), list(gold["thetas"])
    with tp.Context(0) as ctx:
        ac = G.aperture_mass_computer(n, 2.0, fs, ctx=ctx)
        grid, w = ac.normalize_shear(x, y, g)
        assert rel(grid, gold["shears"]) < 1e-13 and rel(w, gold["norm"]) < 1e-13
        assert rel(ac.Map_fft(gold["shears"], norm=gold["norm"]), gold["map_theta2"]) < 1e-11
        acp = G.aperture_mass_computer(n, 2.0, fs, use_polynomial_filter=True, ctx=ctx)
        assert rel(acp.Map_fft(gold["shears"], norm=gold["norm"]), gold["map_theta2_poly"]) < 1e-11
        for poly in (False, True):
            for same in (False, True):
                got = G.extract_Map3_of_field(gold["shears"], n, th, fs, norm=gold["norm"],
                                              same_fieldsize_for_all_theta=same, use_polynomial_filter=poly, ctx=ctx)
                assert rel(got, gold[f"map3_poly{int(poly)}_same{int(same)}"]) < 1e-10, (poly, same)
        got = G.extract_Map3(x, y, g, n, th, fs, ctx=ctx)
        assert rel(got, gold["map3_catalogue"]) < 1e-10


@pytest.mark.gpu
def test_gpu_matches_oracle_other_sizes():
    """A grid whose padded FFT size is not a power of two (npix 100 -> 200),
    four apertures, the cross maps and the convergence path."""
    tp, G = _gpu()
    rng = np.random.default_rng(5)
    n, fs, th = 100, 50.0, [1.0, 1.7, 2.5, 4.0]
    x, y = rng.uniform(0, fs, 8000), rng.uniform(0, fs, 8000)
    g = 0.05 * np.exp(2j * np.pi * x / 17.0) + 0.3 * (rng.standard_normal(8000) + 1j * rng.standard_normal(8000))
    with tp.Context(0) as ctx:
        ref = A.extract_map3(x, y, g, n, th, fs)
        got = G.extract_Map3(x, y, g, n, th, fs, ctx=ctx)
        assert rel(got, ref) < 1e-10
        # six apertures: the general triplet reduction (five or fewer keep
        # their sums in registers)
        th6 = [1.0, 1.4, 1.7, 2.1, 2.5, 3.2]
        assert rel(G.extract_Map3(x, y, g, n, th6, fs, ctx=ctx), A.extract_map3(x, y, g, n, th6, fs)) < 1e-10
        grid, w = A.cic_grid(x, y, g, n, fs)
        ac = G.aperture_mass_computer(n, 2.5, fs, ctx=ctx)
        m, xm = ac.Map_fft(grid, norm=w, return_mcross=True)
        rm, rx = A.map_weighted(grid, w, A.q_grid(n, fs, 2.5), return_cross=True)
        assert rel(m, rm) < 1e-11 and rel(xm, rx) < 1e-11
        kappa = rng.standard_normal((n, n))
        assert rel(ac.Map_fft_from_kappa(kappa), A.map_from_kappa(kappa, n, fs, 2.5)) < 1e-11


@pytest.mark.gpu
def test_gpu_rejects_unsupported_options():
    tp, G = _gpu()
    with tp.Context(0) as ctx:
        ac = G.aperture_mass_computer(32, 2.0, 20.0, ctx=ctx)
        with pytest.raises(ValueError):
            ac.normalize_shear(np.zeros(3), np.zeros(3), np.zeros(3, complex), CIC=False)
        with pytest.raises(ValueError):
            ac.Map_fft(np.zeros((32, 32), complex))
        with pytest.raises(tp.ThreepointError):
            tp.aperture_mass._Plan(ctx, 32, 20.0, [0.0], False)


@pytest.mark.gpu
def test_gpu_fp32_transforms_against_fp64():
    """FP32 transforms and Fourier products (gridding, maps and sums in FP64)
    against the FP64 pipeline: maps within 1e-5 of their largest value, <Map^3>
    within 1e-3."""
    tp, G = _gpu()
    rng = np.random.default_rng(9)
    n, fs, th = 128, 60.0, [1.0, 2.0, 4.0]
    x, y = rng.uniform(0, fs, 20000), rng.uniform(0, fs, 20000)
    g = 0.05 * np.exp(2j * np.pi * (x / 13.0 + y / 29.0)) + 0.3 * (rng.standard_normal(20000) +
                                                                  1j * rng.standard_normal(20000))
    with tp.Context(0) as ctx:
        p64 = G._Plan(ctx, n, fs, th, False, precision=0)
        p32 = G._Plan(ctx, n, fs, th, False, precision=1)
        p64.grid(x, y, g)
        p32.grid(x, y, g)
        m64, m32 = p64.maps(), p32.maps()
        assert rel(m32, m64) < 1e-5
        v64, v32 = p64.map3(True), p32.map3(True)
        assert np.max(np.abs(v32 - v64) / np.abs(v64)) < 1e-3
