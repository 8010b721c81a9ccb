"""Host-side checks that need no GPU: the C ABI exports, the input parsers."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import oracle as O
from conftest import COSMO1, ROOT


@pytest.fixture(scope="module")
def tplib():
    from threepoint_gb300 import build as B

    B.build()
    import threepoint_gb300 as tp

    return tp


def declared_symbols():
    hdrs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]
    syms = set()
    for h in hdrs:
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(tp_[a-z0-9_]+)\s*\(", txt, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_library_exports_every_declared_symbol(tplib):
    L = C.CDLL(tplib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s


def test_param_file_parser(tplib, tmp_path):
    p = tmp_path / "c.param"
    p.write_text("# cosmology\nh 0.6898\nsigma_8 0.826\nOmega_b 0.0473\nn_s 0.969\nw -1\nOmega_m 0.2905\nz_max 3\n")
    c = tplib.cosmology.from_file(str(p))
    ref = O.read_param_file(str(p))
    for k in ("h", "sigma8", "omb", "ns", "w", "om", "zmax", "ow", "omc"):
        assert getattr(c, k) == ref[k]
    bad = tmp_path / "bad.param"
    bad.write_text("h 0.7\nfoo 1\n")
    with pytest.raises(tplib.ThreepointError):
        tplib.cosmology.from_file(str(bad))
    with pytest.raises(tplib.ThreepointError):
        tplib.cosmology.from_file(str(tmp_path / "missing.param"))


def test_read_n_of_z_matches_oracle(tplib, nz_file, nz256):
    nz = tplib.read_n_of_z(nz_file, 256, 3.0)
    assert np.allclose(nz, nz256, rtol=1e-12, atol=0)
    assert abs(nz.sum() * 3.0 / 256 - 1) < 1e-12


def test_read_n_of_z_coarse_file(tplib, tmp_path):
    # a file coarser than the internal bins takes the bin-averaging branch
    zs = np.linspace(0, 3, 101)
    ns = zs ** 2 * np.exp(-zs / 0.4)
    p = tmp_path / "coarse.dat"
    p.write_text("".join(f"{z} {n}\n" for z, n in zip(zs, ns)))
    got = tplib.read_n_of_z(str(p), 256, 3.0)
    ref = O.read_n_of_z(zs, ns, 256, 3.0)
    assert np.allclose(got, ref, rtol=1e-12)


def test_read_thetas_and_units(tplib, tmp_path):
    p = tmp_path / "t.dat"
    p.write_text("# thetas\n2\n4\n8\n16\n")
    t = tplib.read_thetas(str(p))
    assert list(t) == [2, 4, 8, 16]
    assert tplib.convert_angle_to_rad(1, "arcmin") == 2.9088820866e-4
    assert tplib.convert_angle_to_rad(2, "deg") == 2 * 0.017453
    assert len(tplib.theta_triplets(t)) == 20
    with pytest.raises(tplib.ThreepointError):
        tplib.convert_angle_to_rad(1, "furlong")


def test_no_cpu_fallback_without_gpu(tplib):
    """Without a GPU the numerical API fails loudly instead of computing on the CPU."""
    from conftest import gpu_available

    if gpu_available():
        pytest.skip("GPU present")
    with pytest.raises(tplib.ThreepointError):
        tplib.Context(0)
