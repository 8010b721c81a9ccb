"""Host-side checks of the drop-in entry points that need no GPU: the cosmosis
module's setup (options, triplets, errors), the covariance-parameter and
Gamma-config readers, and the command-line drivers' argument handling."""
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def tp():
    from threepoint_gb300 import build as B

    B.build()
    import threepoint_gb300 as tp

    return tp


class FakeBlock:
    """The subset of cosmosis.datablock.DataBlock that the module uses."""

    def __init__(self, values=None):
        self.v = dict(values or {})

    def _get(self, s, k):
        if (s, k) not in self.v:
            raise KeyError((s, k))
        return self.v[s, k]

    def get_double(self, s, k):
        return float(self._get(s, k))

    def get_int(self, s, k):
        v = self._get(s, k)
        if isinstance(v, bool) or not isinstance(v, int):
            raise TypeError(k)
        return v

    def get_bool(self, s, k):
        return bool(self._get(s, k))

    def get_string(self, s, k):
        v = self._get(s, k)
        if not isinstance(v, str):
            raise TypeError(k)
        return v

    def get_double_array_nd(self, s, k):
        return np.asarray(self._get(s, k), dtype=float)

    def put_double_array_1d(self, s, k, a):
        self.v[s, k] = np.asarray(a, dtype=float)


def options(nz, out_dir="", **kw):
    o = {"nz_file": nz, "zMax": 3.0, "theta_unit": "arcmin", "theta_min": 2.0, "theta_max": 16.0,
         "theta_bins": 4, "diag_only": False, "output_Map3": False, "output_dir": str(out_dir)}
    o.update(kw)
    return FakeBlock({("threepoint", k): v for k, v in o.items()})


def reference_triplets(tmin, tmax, nbins, diag):
    """interface.cu:103-133, restated"""
    d = (math.log(tmax) - math.log(tmin)) / (nbins - 1)
    out = []
    for i in range(nbins):
        t1 = tmin * math.exp(i * d)
        if diag:
            out.append((t1, t1, t1))
            continue
        for j in range(i, nbins):
            t2 = tmin * math.exp(j * d)
            for k in range(j, nbins):
                out.append((t1, t2, tmin * math.exp(k * d)))
    return np.array(out)


@pytest.mark.parametrize("diag", [False, True])
def test_module_setup_builds_reference_triplets(tp, nz_file, diag):
    from threepoint_gb300 import cosmosis_module as M

    m = M.setup(options(nz_file, diag_only=diag))
    try:
        got = m.thetas
        arcmin = 2.9088820866e-4
        ref = reference_triplets(2 * arcmin, 16 * arcmin, 4, diag)
        assert got.shape == ref.shape == ((4, 3) if diag else (20, 3))
        assert np.array_equal(got, ref)
    finally:
        M.cleanup(m)


@pytest.mark.parametrize("bad", [dict(theta_unit="parsec"), dict(theta_bins=1), dict(nz_file="/nonexistent/nz.dat"),
                                 dict(zMax="three"), dict(precision="fp16")])
def test_module_setup_errors(tp, nz_file, bad):
    from threepoint_gb300 import cosmosis_module as M

    with pytest.raises((tp.ThreepointError, ValueError)):
        M.setup(options(nz_file, **bad))


def test_module_setup_missing_key(tp, nz_file):
    from threepoint_gb300 import cosmosis_module as M

    o = options(nz_file)
    del o.v["threepoint", "output_dir"]
    with pytest.raises(tp.ThreepointError):
        M.setup(o)


def test_cov_params_reader(tp, tmp_path):
    # the layout of the reference's example covariance parameter file
    p = tmp_path / "cov_param.dat"
    p.write_text("#Example covariance param file\n\n# Survey Side length [unit]\nthetaMax 7.87\n\n"
                 "shapenoise_sigma 0.3\n\ngalaxy_density 167772.16\n\nunit deg\n\nshapenoiseOnly 1\n"
                 "area 61.9369\nthetaMax_smaller 3.5\n")
    c = tp.covarianceParameters.from_file(str(p))
    deg = 0.017453  # convert_angle_to_rad(1, "deg") (helpers.cu:130-153)
    assert c.theta_max == 7.87 * deg
    assert c.theta_max_smaller == 3.5 * deg
    assert c.shapenoise_sigma == 0.3
    assert c.galaxy_density == 167772.16 / deg / deg
    assert c.area == 61.9369 * deg * deg
    assert c.shapenoise_only is True
    bad = tmp_path / "bad.dat"
    bad.write_text("thetaMax 1\nunit furlong\n")
    with pytest.raises(tp.ThreepointError):
        tp.covarianceParameters.from_file(str(bad))
    bad.write_text("thetaMax 1\nunit deg\nfoo 2\n")
    with pytest.raises(tp.ThreepointError):
        tp.covarianceParameters.from_file(str(bad))


def test_gamma_config_and_triangles(tp, tmp_path):
    p = tmp_path / "gamma.param"
    p.write_text("# binning\nrmin 0.1\nrmax 100\numin 0\numax 1\nvmin -1\nvmax 1\nrsteps 10\nusteps 10\nvsteps 10\n")
    cfg = tp.configGamma.from_file(str(p))
    assert (cfg.rsteps, cfg.usteps, cfg.vsteps) == (10, 10, 10)
    x, ruv = cfg.triangles()
    assert x.shape == (1000, 3)
    # calculateGamma.cu:104-121, restated
    lr0, lr1 = math.log(0.1), math.log(100)
    t = 0
    for i in range(10):
        r = math.exp(lr0 + (lr1 - lr0) / 10 * (i + 0.5))
        for j in range(10):
            u = 0 + 1 / 10 * (j + 0.5)
            for k in range(10):
                v = -1 + 2 / 10 * (k + 0.5)
                r2 = r * math.pi / 180 / 60
                r3 = r2 * u
                assert tuple(x[t]) == (v * r3 + r2, r2, r3)
                assert tuple(ruv[t]) == (r, u, v)
                t += 1
    # every bin centre is a proper triangle
    a, b, c = x.T
    assert np.all(a <= b + c) and np.all(b <= a + c) and np.all(c <= a + b)
    p.write_text("rmin 0.1\n")
    with pytest.raises(tp.ThreepointError):
        tp.configGamma.from_file(str(p))


def _run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("name,nargs", [("calculateApertureStatistics", 3), ("calculateGamma", 3),
                                        ("calculateApertureStatisticsCovariance", 12)])
def test_driver_usage_on_wrong_argc(tp, name, nargs):
    from threepoint_gb300 import build as B

    r = _run(B.driver(name), *(["x"] * nargs))
    assert r.returncode != 0
    assert "Wrong number of command line parameters" in r.stderr


@pytest.mark.parametrize("flags,geometry,message", [
    ((0, 0, 1, 0, 0, 0, 0), "square", "T4: Wrong survey geometry"),
    ((0, 0, 0, 1, 0, 0, 0), "square", "T5: Wrong survey geometry"),
    ((0, 0, 0, 0, 1, 0, 0), "circle", "T6: Wrong survey geometry"),
    ((1, 0, 0, 0, 0, 1, 0), "rectangular", "T7: Wrong survey geometry"),
    ((0, 0, 0, 0, 0, 0, 1), "circle", "T7_SSC: Wrong survey geometry"),
])
def test_cov_driver_checks_term_geometries(tp, tmp_path, flags, geometry, message):
    """Terms coded for some survey geometries only fail before any output, as
    the reference's driver does when the term throws at the first pair."""
    from threepoint_gb300 import build as B

    p = tmp_path / "cov.param"
    p.write_text("thetaMax 10\nshapenoise_sigma 0.3\ngalaxy_density 10\nunit arcmin\nshapenoiseOnly 1\narea 100\n")
    out = tmp_path / "out"
    out.mkdir()
    r = _run(B.driver("calculateApertureStatisticsCovariance"), "c", "t", "nz", str(out) + "/", p, *flags, geometry)
    assert r.returncode != 0
    assert message in r.stderr
    assert not os.listdir(out)


def test_cov_driver_rejects_unknown_geometry(tp, tmp_path):
    from threepoint_gb300 import build as B

    p = tmp_path / "cov.param"
    p.write_text("thetaMax 10\nshapenoise_sigma 0.3\ngalaxy_density 10\nunit arcmin\nshapenoiseOnly 1\narea 100\n")
    r = _run(B.driver("calculateApertureStatisticsCovariance"), "c", "t", "nz", str(tmp_path) + "/", p,
             1, 0, 0, 0, 0, 0, 0, "hexagon")
    assert r.returncode != 0
    assert "Cov type not correctly specified" in r.stderr
