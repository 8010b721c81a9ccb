"""The drop-in entry points on the GPU: the cosmosis module (setup / execute /
cleanup over a fake data block) against the oracle, and the three
command-line drivers against the library calls they batch, with the
reference's output formats."""
import math
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import COSMO1
from test_host_drivers import FakeBlock, options

pytestmark = pytest.mark.gpu
ARC = O.ARCMIN


def convert_pk(k, p, n=256):
    """convert_Pk + valueMap (cuda_version/helpers.cu:202-235), restated."""
    kmin, kmax = k[0], k[-1]
    dk = math.log(kmax / kmin) / n
    out = []
    for i in range(n):
        kk = math.exp(math.log(kmin) + dk * i)
        hi = int(np.searchsorted(k, kk, side="right"))
        if hi == len(k):
            out.append(p[-1])
        elif hi == 0:
            out.append(p[0])
        else:
            d = (kk - k[hi - 1]) / (k[hi] - k[hi - 1])
            out.append(d * p[hi] + (1 - d) * p[hi - 1])
    return np.array(out), dk, kmin, kmax


@pytest.fixture(scope="module")
def lin_pk(oracle_tables):
    k = np.exp(np.linspace(np.log(1e-4), np.log(1e2), 300))
    p = np.array([oracle_tables.linear_pk(x) for x in k])
    return k, p


def cosmo_block(k, p, **over):
    c = dict(omega_m=COSMO1["om"], sigma_8=COSMO1["sigma8"], h0=COSMO1["h"], omega_b=COSMO1["omb"],
             n_s=COSMO1["ns"], w=COSMO1["w"])
    c.update(over)
    v = {("cosmological_parameters", n): x for n, x in c.items()}
    v["matter_power_lin", "k_h"] = k
    # two redshift rows: the module reads the first (interface.cu:185-188)
    v["matter_power_lin", "p_k"] = np.stack([p, 3 * p])
    return FakeBlock(v)


def test_module_execute_matches_oracle(nz_file, nz256, lin_pk, tmp_path):
    from threepoint_gb300 import cosmosis_module as M

    k, p = lin_pk
    m = M.setup(options(nz_file, tmp_path, theta_min=8.0, theta_max=16.0, theta_bins=2, diag_only=True,
                        output_Map3=True))
    try:
        blk = cosmo_block(k, p)
        assert M.execute(blk, m) == 0
        got = blk.v["threepoint", "Map3s"]
        pk, dk, kmin, kmax = convert_pk(k, p)
        T = O.Tables(COSMO1, nz256, pk, dk, kmin, kmax)
        O.set_threads(0)
        for th, g in zip(m.thetas, got):
            ref = T.map3(list(th))[0]
            assert g == pytest.approx(ref, rel=1e-6)
        fn = tmp_path / "om_0.300000_sig8_0.800000_h_0.700000_w_-1.000000.dat"
        lines = fn.read_text().splitlines()
        assert lines[0] == "#theta1[rad] theta2[rad] theta3[rad] Map^3"
        assert len(lines) == 3 and all(len(x.split()) == 4 for x in lines[1:])
        assert float(lines[1].split()[3]) == pytest.approx(got[0], rel=1e-5)
        # a second cosmology through the same module object: more power
        # (larger sigma_8 and P(k)) gives a larger <Map^3>
        blk2 = cosmo_block(k, 1.21 * p, sigma_8=0.88)
        M.execute(blk2, m)
        assert np.all(blk2.v["threepoint", "Map3s"] > got)
    finally:
        M.cleanup(m)


def test_module_fp32(nz_file, lin_pk):
    from threepoint_gb300 import cosmosis_module as M

    k, p = lin_pk
    o = options(nz_file, theta_min=4.0, theta_max=16.0, theta_bins=3, diag_only=False)
    m64 = M.setup(o)
    o.v["threepoint", "precision"] = "fp32"
    m32 = M.setup(o)
    try:
        b64, b32 = cosmo_block(k, p), cosmo_block(k, p)
        M.execute(b64, m64)
        M.execute(b32, m32)
        a, b = b64.v["threepoint", "Map3s"], b32.v["threepoint", "Map3s"]
        assert len(a) == 10
        assert np.max(np.abs(b / a - 1)) < 1e-3
    finally:
        M.cleanup(m64)
        M.cleanup(m32)


# ---------------------------------------------------------------------------
def _write_inputs(d, nz_file):
    cos = d / "cosmo.dat"
    cos.write_text("# cosmology\nh {h}\nsigma_8 {sigma8}\nOmega_b {omb}\nn_s {ns}\nw {w}\nOmega_m {om}\n"
                   "z_max {zmax}\n".format(**COSMO1))
    th = d / "thetas.dat"
    th.write_text("8\n16\n")
    return str(cos), str(th), nz_file


def _run(name, *args):
    from threepoint_gb300 import build as B

    r = subprocess.run([B.driver(name), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r


def test_driver_map3(gpu_ctx, nz_file, tmp_path):
    cos, th, nz = _write_inputs(tmp_path, nz_file)
    out = tmp_path / "map3.dat"
    _run("calculateApertureStatistics", cos, th, out, nz)
    lines = out.read_text().splitlines()
    trip = [(8, 8, 8), (8, 8, 16), (8, 16, 16), (16, 16, 16)]
    assert len(lines) == 4
    ref = gpu_ctx.map3_batch(np.array(trip) * ARC, [0])[0]
    for ln, t, r in zip(lines, trip, ref):
        assert ln.endswith(" ")  # "t1 t2 t3 Map3 " (calculateApertureStatistics.cu:124-125)
        v = ln.split()
        assert tuple(int(x) for x in v[:3]) == t
        assert float(v[3]) == pytest.approx(r, rel=1e-5)  # 6 significant digits in the file


def test_driver_gamma(gpu_ctx, nz_file, tmp_path):
    cos, _, nz = _write_inputs(tmp_path, nz_file)
    cfg = tmp_path / "gamma.param"
    cfg.write_text("rmin 1\nrmax 10\numin 0.5\numax 1\nvmin 0\nvmax 0.5\nrsteps 1\nusteps 1\nvsteps 2\n")
    out = tmp_path / "gamma.dat"
    _run("calculateGamma", cos, cfg, out, nz)
    lines = out.read_text().splitlines()
    assert len(lines) == 2
    import threepoint_gb300 as tp

    x, ruv = tp.configGamma.from_file(str(cfg)).triangles()
    ref = gpu_ctx.gamma_batch(x)
    for ln, g, q in zip(lines, ref, ruv):
        v = [float(s) for s in ln.split()]
        assert len(v) == 11
        got = np.array(v[0:8:2]) + 1j * np.array(v[1:8:2])
        assert np.allclose(got, g, rtol=1e-5, atol=1e-5 * np.abs(g).max())
        assert v[8:] == pytest.approx(list(q), rel=1e-5)


def test_driver_covariance(nz_file, tmp_path):
    import threepoint_gb300 as tp

    cos, th, nz = _write_inputs(tmp_path, nz_file)
    th_file = tmp_path / "thetas1.dat"
    th_file.write_text("8\n")
    par = tmp_path / "cov_param.dat"
    par.write_text("thetaMax 10\nshapenoise_sigma 0.3\ngalaxy_density 36000\nunit deg\nshapenoiseOnly 1\n"
                   "area 100\n")
    outdir = tmp_path / "out"
    outdir.mkdir()
    _run("calculateApertureStatisticsCovariance", cos, th_file, nz, str(outdir) + "/", par, 1, 1, 0, 0, 0, 0, 0,
         "infinite")
    cp = tp.covarianceParameters.from_file(str(par))
    n_deg = cp.galaxy_density / 57.3 / 57.3
    name = "cov_infinite_term1Numerical_sigma_0.30_n_{:.2f}_thetaMax_{:.2f}_gpu.dat".format(n_deg, cp.theta_max * 57.3)
    f1 = outdir / name
    assert f1.exists(), os.listdir(outdir)
    assert (outdir / name.replace("term1", "term2")).exists()
    v1 = [float(x) for x in f1.read_text().split()]
    assert len(v1) == 1
    ctx = tp.Context(0)
    ctx.set_shape_noise(cp.shapenoise_sigma, cp.galaxy_density, True)
    ctx.set_cosmology(tp.cosmology.from_file(cos), tp.read_n_of_z(nz, 256, COSMO1["zmax"]))
    t = np.array([[8 * ARC] * 3])
    ref = ctx.cov_total(1, t, t, geometry=tp.GEOM_INFINITE, thetaMax=cp.theta_max, area=cp.area)[0]
    ctx.close()
    assert v1[0] == pytest.approx(ref, rel=1e-5)
    # T2 of an infinite survey is 0
    assert [float(x) for x in (outdir / name.replace("term1", "term2")).read_text().split()] == [0.0]


def test_driver_covariance_matrix_layout(nz_file, tmp_path):
    """Two radii -> 4 triplets -> a symmetric 4 x 4 matrix, writeCov's layout."""
    cos, th, nz = _write_inputs(tmp_path, nz_file)
    par = tmp_path / "cov_param.dat"
    par.write_text("thetaMax 10\nshapenoise_sigma 0.3\ngalaxy_density 36000\nunit deg\nshapenoiseOnly 1\n"
                   "area 100\n")
    outdir = tmp_path / "out"
    outdir.mkdir()
    _run("calculateApertureStatisticsCovariance", cos, th, nz, str(outdir) + "/", par, 1, 0, 0, 0, 0, 0, 0,
         "infinite")
    (f,) = list(outdir.iterdir())
    rows = f.read_text().splitlines()
    assert len(rows) == 4 and all(r.endswith(" ") for r in rows)
    m = np.array([[float(x) for x in r.split()] for r in rows])
    assert np.array_equal(m, m.T)
    assert np.all(np.diag(m) > 0)


def test_driver_covariance_halo_terms(nz_file, tmp_path):
    """T7 and T7_2h through the covariance driver: one radius -> one entry;
    T7 equals the library's FP32 node sums (the driver's fp32 argument) and
    T7_2h is the reference's zero."""
    import threepoint_gb300 as tp

    cos, th, nz = _write_inputs(tmp_path, nz_file)
    th_file = tmp_path / "thetas1.dat"
    th_file.write_text("8\n")
    par = tmp_path / "cov_param.dat"
    par.write_text("thetaMax 10\nshapenoise_sigma 0.3\ngalaxy_density 36000\nunit deg\nshapenoiseOnly 0\n"
                   "area 100\n")
    outdir = tmp_path / "out"
    outdir.mkdir()
    _run("calculateApertureStatisticsCovariance", cos, th_file, nz, str(outdir) + "/", par, 0, 0, 0, 0, 0, 1, 1,
         "infinite", "fp32")
    cp = tp.covarianceParameters.from_file(str(par))
    n_deg = cp.galaxy_density / 57.3 / 57.3
    name = "cov_infinite_term7Numerical_sigma_0.30_n_{:.2f}_thetaMax_{:.2f}_gpu.dat".format(n_deg, cp.theta_max * 57.3)
    v7 = [float(x) for x in (outdir / name).read_text().split()]
    v72 = [float(x) for x in (outdir / name.replace("term7Numerical", "term7_2h_Numerical")).read_text().split()]
    assert v72 == [0.0]
    ctx = tp.Context(0)
    ctx.set_shape_noise(cp.shapenoise_sigma, cp.galaxy_density, False)
    ctx.set_cosmology(tp.cosmology.from_file(cos), tp.read_n_of_z(nz, 256, COSMO1["zmax"]))
    t = np.array([[8 * ARC] * 3])
    ref = ctx.cov_total(7, t, t, geometry=tp.GEOM_INFINITE, thetaMax=cp.theta_max, area=cp.area, precision=1)[0]
    ctx.close()
    assert len(v7) == 1 and v7[0] != 0
    assert v7[0] == pytest.approx(ref, rel=1e-5)
