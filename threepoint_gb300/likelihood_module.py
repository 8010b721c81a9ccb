"""cosmosis likelihood module of threepoint_gb300: ``setup`` / ``execute`` / ``cleanup``.

Drop-in for the reference's likelihood module (cosmosis/threepoint_likelihood.py,
section ``threepoint_likelihood`` in cosmosis/pipeline_gpu.ini:58-63): reads the
measured <Map^3> (4th column of ``data``) and the covariance (last column of
``cov_mat``, reshaped N x N), writes C^-1 to ``cov_inv`` as the reference does,
and stores log L = -chi2/2 of ``threepoint/Map3s`` in
``likelihoods/threepoint_likelihood_LIKE``. The covariance is factored and
chi2 evaluated on the GPU (threepoint_gb300.Likelihood).
"""
from __future__ import annotations

import numpy as np

from . import Likelihood

SECTION = "threepoint_likelihood"


def _get(block, section, key):
    try:
        return block[section, key]
    except Exception:
        return block.get_string(section, key)


def setup(options):
    fn_data = _get(options, SECTION, "data")
    fn_cov = _get(options, SECTION, "cov_mat")
    fn_cov_inv = _get(options, SECTION, "cov_inv")
    data = np.loadtxt(fn_data, comments="#")[:, 3]
    cov = np.loadtxt(fn_cov, comments="#")[:, -1]
    n = len(data)
    lk = Likelihood(data, cov.reshape((n, n)))
    np.savetxt(fn_cov_inv, lk.cov_inv())
    return lk


def execute(block, config):
    model = np.asarray(block["threepoint", "Map3s"], dtype=np.float64)
    block["likelihoods", "threepoint_likelihood_LIKE"] = float(config.loglike(model)[0])
    return 0


def cleanup(config):
    config.close()
