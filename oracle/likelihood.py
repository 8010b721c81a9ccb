"""CPU restatement of the reference's likelihood module for the tests (test
infrastructure, not part of the product): cosmosis/threepoint_likelihood.py:17-27
(covariance read and numpy inverse) and :44-54 (chi2 and log-likelihood)."""
import numpy as np


def cov_inv(cov):
    return np.linalg.inv(np.asarray(cov, dtype=np.float64))


def loglike(model, data, cov):
    r = np.asarray(model, dtype=np.float64) - np.asarray(data, dtype=np.float64)
    chi2 = r.dot(cov_inv(cov)).dot(r)
    log_det = 0
    return -0.5 * (chi2 + log_det)
