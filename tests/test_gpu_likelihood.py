"""The likelihood consumer on the GPU against the CPU restatement of the
reference's cosmosis likelihood module (oracle/likelihood.py)."""
import numpy as np
import pytest

from oracle import likelihood as OL
from test_host_drivers import FakeBlock

pytestmark = pytest.mark.gpu


def spd(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(n, n))
    c = a @ a.T / n + np.diag(rng.uniform(0.5, 2.0, n))
    return c * 1e-20  # <Map^3>^2-like magnitudes


@pytest.fixture(scope="module")
def problem():
    n = 220
    cov = spd(n, 1)
    rng = np.random.default_rng(2)
    data = rng.normal(size=n) * 1e-10
    models = data + rng.normal(size=(64, n)) * 1e-10
    return data, cov, models


def test_chi2_matches_oracle(problem):
    import threepoint_gb300 as tp

    data, cov, models = problem
    lk = tp.Likelihood(data, cov)
    got = lk.loglike(models)
    ref = np.array([OL.loglike(m, data, cov) for m in models])
    assert np.allclose(got, ref, rtol=1e-9, atol=0)
    inv = lk.cov_inv()
    ref_inv = OL.cov_inv(cov)
    assert np.linalg.norm(inv - ref_inv) / np.linalg.norm(ref_inv) < 1e-9
    lk.close()


def test_chi2_device_strided(problem):
    import torch

    import threepoint_gb300 as tp

    data, cov, models = problem
    lk = tp.Likelihood(data, cov)
    n = len(data)
    dev = torch.zeros((len(models), n + 7), dtype=torch.float64, device="cuda")
    dev[:, :n] = torch.tensor(models, device="cuda")
    out = torch.zeros(len(models), dtype=torch.float64, device="cuda")
    lk.chi2_device(dev, out)
    torch.cuda.synchronize()
    assert np.allclose(out.cpu().numpy(), lk.chi2(models), rtol=1e-12, atol=0)


def test_not_positive_definite_is_rejected():
    import threepoint_gb300 as tp

    c = np.eye(5)
    c[2, 2] = -1.0
    with pytest.raises(tp.ThreepointError):
        tp.Likelihood(np.zeros(5), c)
    with pytest.raises(tp.ThreepointError):
        tp.Likelihood(np.zeros(3), np.full((3, 3), np.nan))


def test_small_and_identity():
    import threepoint_gb300 as tp

    lk = tp.Likelihood([1.0], [[4.0]])
    assert lk.chi2([[3.0]])[0] == pytest.approx(1.0, rel=1e-15)
    lk2 = tp.Likelihood(np.zeros(3), np.eye(3))
    assert lk2.chi2([[1.0, 2.0, 2.0]])[0] == pytest.approx(9.0, rel=1e-15)


def test_cosmosis_likelihood_module(problem, tmp_path):
    from threepoint_gb300 import likelihood_module as LM

    data, cov, models = problem
    n = len(data)
    # the reference's file layouts: data column 3, covariance last column
    np.savetxt(tmp_path / "data.dat", np.column_stack([np.zeros(n), np.zeros(n), np.zeros(n), data]),
               header="theta1 theta2 theta3 Map3")
    ij = np.array([(i, j) for i in range(n) for j in range(n)])
    np.savetxt(tmp_path / "cov.dat", np.column_stack([ij, cov.reshape(-1)]))
    opts = FakeBlock({("threepoint_likelihood", "data"): str(tmp_path / "data.dat"),
                      ("threepoint_likelihood", "cov_mat"): str(tmp_path / "cov.dat"),
                      ("threepoint_likelihood", "cov_inv"): str(tmp_path / "cov_inv.dat")})
    cfg = LM.setup(_Indexable(opts))
    inv = np.loadtxt(tmp_path / "cov_inv.dat")
    cov_f = np.loadtxt(tmp_path / "cov.dat")[:, -1].reshape(n, n)
    assert np.linalg.norm(inv - OL.cov_inv(cov_f)) / np.linalg.norm(inv) < 1e-9
    blk = _Indexable(FakeBlock({("threepoint", "Map3s"): models[0]}))
    assert LM.execute(blk, cfg) == 0
    data_f = np.loadtxt(tmp_path / "data.dat")[:, 3]
    assert blk.b.v["likelihoods", "threepoint_likelihood_LIKE"] == pytest.approx(
        OL.loglike(models[0], data_f, cov_f), rel=1e-9)
    LM.cleanup(cfg)


class _Indexable:
    """block[section, key] access over the fake block (cosmosis DataBlock style)."""

    def __init__(self, b):
        self.b = b

    def __getitem__(self, k):
        return self.b._get(*k)

    def __setitem__(self, k, v):
        self.b.v[k] = v

    def get_string(self, s, k):
        return self.b.get_string(s, k)
