import math
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


# Config-1 cosmology and source distribution: flat wCDM, n(z) ~ z^2 exp(-(z/0.5)^1.5)
# on 0<z<3 tabulated at dz=1e-3 and rebinned to 256 bins by read_n_of_z.
COSMO1 = dict(h=0.7, sigma8=0.8, omb=0.048, ns=0.96, w=-1.0, om=0.3, zmax=3.0)
COSMO1["ow"] = 1 - COSMO1["om"]
COSMO1["omc"] = COSMO1["om"] - COSMO1["omb"]


def nz_table():
    zs = np.arange(3001) * 1e-3
    ns = zs ** 2 * np.exp(-(zs / 0.5) ** 1.5)
    return zs, ns


@pytest.fixture(scope="session")
def nz_file(tmp_path_factory):
    d = tmp_path_factory.mktemp("inputs")
    p = d / "nz_config1.dat"
    zs, ns = nz_table()
    with open(p, "w") as f:
        f.write("# z n(z)\n")
        for z, n in zip(zs, ns):
            f.write(f"{z:.6f} {n:.17g}\n")
    return str(p)


@pytest.fixture(scope="session")
def nz256():
    import oracle

    zs, ns = nz_table()
    return oracle.read_n_of_z(zs, ns, 256, 3.0)


@pytest.fixture(scope="session")
def oracle_tables(nz256):
    import oracle

    return oracle.Tables(COSMO1, nz256)


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx(nz256):
    if not gpu_available():
        pytest.skip("no CUDA device")
    import threepoint_gb300 as tp

    ctx = tp.Context(0)
    ctx.set_cosmology(tp.cosmology(**COSMO1), nz256)
    yield ctx
    ctx.close()
