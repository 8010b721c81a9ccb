"""The reference's C++ API over the C ABI (include/threepoint_gb300_compat.hpp):
a C++ caller written against it compiles and links here (CPU), and its values
equal the Python API's on the GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import COSMO1, ROOT

HERE = os.path.dirname(os.path.abspath(__file__))


def build_example(tmpdir):
    from threepoint_gb300 import build as B

    B.build()
    exe = os.path.join(str(tmpdir), "compat_example")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
           os.path.join(HERE, "compat", "compat_example.cpp"), "-L" + B.BUILD, "-lthreepoint_gb300",
           "-Wl,-rpath," + B.BUILD, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compat_header_compiles_and_links(tmp_path):
    exe = build_example(tmp_path)
    assert os.path.exists(exe)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2  # usage: no GPU call made


@pytest.mark.gpu
def test_compat_values_match_python_api(tmp_path, nz_file, nz256):
    import threepoint_gb300 as tp

    exe = build_example(tmp_path)
    par = tmp_path / "cosmo.param"
    par.write_text("h {h}\nsigma_8 {sigma8}\nOmega_b {omb}\nn_s {ns}\nw {w}\nOmega_m {om}\nz_max {zmax}\n".format(**COSMO1))
    r = subprocess.run([exe, str(par), nz_file], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    m3, g_re, g_im, t2 = (float(v) for v in r.stdout.split())
    arc = 2.9088820866e-4
    a, b = 8 * arc, 16 * arc
    ctx = tp.Context(0)
    ctx.set_cosmology(tp.cosmology(**COSMO1), tp.read_n_of_z(nz_file, 256, COSMO1["zmax"]))
    assert m3 == pytest.approx(ctx.MapMapMap([a, a, b]), rel=1e-12)
    g = ctx.gamma0(a, a, 0.5 * a)
    assert g_re == pytest.approx(g.real, rel=1e-12, abs=1e-30)
    assert g_im == pytest.approx(g.imag, rel=1e-12, abs=1e-30)
    tmax = 10 * 0.017453
    ctx.set_shape_noise(0.3, 10 / arc ** 2, True)
    ref = ctx.T2_total([a, a, b], [a, b, b], geometry=tp.GEOM_SQUARE, thetaMax=tmax, area=tmax * tmax)
    assert t2 == pytest.approx(ref, rel=1e-12)
    ctx.close()


def test_t7_2h_total_is_the_references_zero():
    """T7_2h of the reference is 0 for the square and infinite surveys (its
    integrand's variance table is never filled) and throws for the others."""
    import threepoint_gb300 as tp

    a, b = [1e-3] * 3, [2e-3] * 3
    assert tp.Context.T7_2h_total(a, b, geometry=tp.GEOM_SQUARE) == 0.0
    assert tp.Context.T7_2h_total(a, b, geometry=tp.GEOM_INFINITE) == 0.0
    for g in (tp.GEOM_CIRCLE, tp.GEOM_RECTANGLE):
        with pytest.raises(ValueError):
            tp.Context.T7_2h_total(a, b, geometry=g)

