"""Brute-force <Map^3> covariance of a Gaussian white-noise convergence field
(test infrastructure, not part of the product): the real-space computation of
classed_version/testCalculateCovarianceGaussianWhiteNoise.cpp restated.

Pixels of side d carry independent convergence values of standard deviation
sigma; the aperture mass at theta_i is sum_k d^2 U(|theta_i - theta_k|) kappa_k
with U(r) = (1 - x) exp(-x) / (2 pi theta^2), x = r^2 / (2 theta^2); the
estimator averages Map^3 over an N x N grid of aperture centres (side L = N d)
in an unbounded noise field. Wick's theorem gives the covariance of two such
estimators as T1 (6 pairings across the two triplets) + T2 (9 pairings: one pair
inside each triplet and one across), with
<Map_a(theta_i) Map_b(theta_j)> = (d^2 sigma)^2 A_ab(theta_j - theta_i),
A_ab = U_a correlated with U_b on the pixel grid (computed by FFT), and the
sum over centre pairs collapsed to separations weighted by their counts
(N - |dx|)(N - |dy|). In the continuum this is the square-window T1_total and
T2_total of apertureStatisticsCovariance.cu with P(ell) = sigma^2 d^2.
"""
import numpy as np


def _U(r, th):
    x = (r / th) ** 2 / 2
    return np.exp(-x) * (1 - x) / (2 * np.pi * th * th)


def t1_t2(th123, th456, side, pix, sigma):
    """(T1, T2) of the estimators for triplets th123, th456 [rad], centre grid
    of side `side` [rad] with pixel `pix` [rad], per-pixel sigma."""
    ths = list(th123) + list(th456)
    m = int(np.ceil(7 * max(ths) / pix))
    g = np.arange(-m, m + 1) * pix
    X, Y = np.meshgrid(g, g, indexing="ij")
    R = np.hypot(X, Y)
    n = 2 * (2 * m + 1)
    F = [np.fft.rfft2(_U(R, t), s=(n, n)) for t in ths]
    cache = {}

    def corr(a, b):
        if (a, b) not in cache:
            cache[a, b] = np.fft.fftshift(np.fft.irfft2(F[a] * np.conj(F[b]), s=(n, n)))
        return cache[a, b]

    nin = int(round(side / pix))
    c0 = n // 2
    w1 = np.clip(nin - np.abs(np.arange(n) - c0), 0, None).astype(float)
    W = np.outer(w1, w1)
    norm = (pix * pix * sigma) ** 6 / nin ** 4
    t1 = sum(np.sum(W * corr(0, p) * corr(1, q) * corr(2, r))
             for p, q, r in [(3, 4, 5), (3, 5, 4), (4, 5, 3), (4, 3, 5), (5, 3, 4), (5, 4, 3)])
    t2 = sum(corr(a, b)[c0, c0] * corr(e, f)[c0, c0] * np.sum(W * corr(c, h))
             for a, b, c in [(0, 1, 2), (0, 2, 1), (1, 2, 0)] for e, f, h in [(3, 4, 5), (3, 5, 4), (4, 5, 3)])
    return t1 * norm, t2 * norm
