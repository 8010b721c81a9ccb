"""FFT aperture-mass measurement, numpy/scipy restatement.

TEST INFRASTRUCTURE ONLY (the checker of threepoint_gb300.aperture_mass).
Restates python_scripts/aperture_mass_computer.py of the reference:
cloud-in-cell gridding of a shear catalogue (normalize_shear with CIC,
:288-372), the Q and U filter grids (Qfunc/Ufunc/Qfunc_array/Ufunc_array,
:72-114), the weighted aperture-mass map (Map_fft with a weight grid,
normalize_weighted and zero padding, :199-286; norm_fft :283-286), the map
from a convergence grid (Map_fft_from_kappa, :183-197) and <Map^3> over the
map interiors (extract_Map3_of_field, :466-531). Pinned against the
reference module itself by tests/golden/reference_apm.npz.
"""
from __future__ import annotations

import numpy as np
from scipy.signal import fftconvolve


def cic_grid(x, y, g, npix, fieldsize):
    """Shear-sum and weight grids [x bin][y bin]: each galaxy adds its
    bilinear cell weights to the numpy.histogram2d bins of (x, y), (x + c, y),
    (x, y + c) and (x + c, y + c), c = fieldsize / (npix - 1), over the edges
    i / (npix - 1) * fieldsize, i = 0..npix."""
    cell = fieldsize / (npix - 1)
    edges = np.arange(npix + 1) / (npix - 1) * fieldsize
    fx, fy = x / cell, y / cell
    dx, dy = fx - np.floor(fx), fy - np.floor(fy)
    re = np.zeros((npix, npix))
    im = np.zeros((npix, npix))
    w = np.zeros((npix, npix))
    for ox, oy, wt in ((0.0, 0.0, (1 - dx) * (1 - dy)), (cell, 0.0, dx * (1 - dy)),
                       (0.0, cell, (1 - dx) * dy), (cell, cell, dx * dy)):
        px, py = x + ox, y + oy
        re += np.histogram2d(px, py, bins=edges, weights=g.real * wt)[0]
        im += np.histogram2d(px, py, bins=edges, weights=g.imag * wt)[0]
        w += np.histogram2d(px, py, bins=edges, weights=wt)[0]
    return re + 1j * im, w


def _offsets(npix, fieldsize):
    i, j = np.indices((npix, npix))
    z = (i - npix / 2) + 1j * (j - npix / 2)
    return z, np.abs(z) * fieldsize / npix


def q_grid(npix, fieldsize, theta, polynomial=False):
    """Q(|z|) conj(z)^2 / |z|^2 on the pixel offsets z from the grid centre
    npix/2 (0 at the centre)."""
    z, r = _offsets(npix, fieldsize)
    t2 = (r / theta) ** 2
    if polynomial:
        Q = np.where(t2 > 1, 0.0, 6 / np.pi * t2 ** 2 * (1 - t2 ** 2)) / theta ** 2
    else:
        Q = t2 / (4 * np.pi * theta ** 2) * np.exp(-t2 / 2)
    out = np.zeros((npix, npix), dtype=complex)
    nz = r != 0
    out[nz] = Q[nz] * np.conj(z[nz]) ** 2 / np.abs(z[nz]) ** 2
    return out


def u_grid(npix, fieldsize, theta):
    _, r = _offsets(npix, fieldsize)
    xh = (r / theta) ** 2 / 2
    return np.exp(-xh) * (1 - xh) / (2 * np.pi) / theta ** 2


def map_weighted(grid, weight, q, return_cross=False):
    """(Im g * Im Q - Re g * Re Q) / (w * |Q|), '*' = fftconvolve 'same'."""
    den = fftconvolve(weight, np.abs(q), "same")
    m = (fftconvolve(grid.imag, q.imag, "same") - fftconvolve(grid.real, q.real, "same")) / den
    if not return_cross:
        return m
    x = -(fftconvolve(grid.real, q.imag, "same") + fftconvolve(grid.imag, q.real, "same")) / den
    return m, x


def map_from_kappa(kappa, npix, fieldsize, theta):
    return fftconvolve(kappa, u_grid(npix, fieldsize, theta), "same") * fieldsize ** 2 / npix ** 2


def border(theta, fieldsize, npix, polynomial=False):
    return int(np.round(theta / fieldsize * npix * (1.0 if polynomial else 4.0)))


def map3_of_maps(maps, thetas, fieldsize, same_fieldsize=False, polynomial=False):
    """Mean of M_i M_j M_k over [c, npix - c)^2 for every i <= j <= k, c the
    border of theta_k (or of the largest aperture)."""
    npix = maps.shape[1]
    tmax = max(thetas)
    out = []
    n = len(thetas)
    for i in range(n):
        for j in range(i, n):
            for k in range(j, n):
                c = border(tmax if same_fieldsize else thetas[k], fieldsize, npix, polynomial)
                sl = slice(c, npix - c)
                out.append(np.mean(maps[i][sl, sl] * maps[j][sl, sl] * maps[k][sl, sl]))
    return np.array(out)


def extract_map3(x, y, g, npix, thetas, fieldsize, same_fieldsize=True, polynomial=False):
    grid, w = cic_grid(x, y, g, npix, fieldsize)
    maps = np.array([map_weighted(grid, w, q_grid(npix, fieldsize, t, polynomial)) for t in thetas])
    return map3_of_maps(maps, thetas, fieldsize, same_fieldsize, polynomial)
