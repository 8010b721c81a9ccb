"""FFT aperture-mass measurement on the GPU, with the interface of the
reference's python_scripts/aperture_mass_computer.py.

    ac = aperture_mass_computer(npix, theta_ap, fieldsize)      # :29-58
    shears, norm = ac.normalize_shear(Xs, Ys, shear_catalogue)  # :288-372 (CIC)
    m = ac.Map_fft(shears, norm=norm)                           # :199-286
    k = ac.Map_fft_from_kappa(kappa)                            # :183-197
    extract_Map3(Xs, Ys, shear_catalogue, npix, thetas, fieldsize)              # :375-405
    extract_Map3_of_field(shears, npix, thetas, fieldsize, norm=norm)           # :407-531

Positions, field size and aperture radii are in arcmin as in the reference;
grids are numpy arrays [x bin][y bin]. The work runs in the C ABI's tp_apm_*
calls (tp_apm.cu): gridding, filters, Fourier products, crop and the triplet
reduction are this library's kernels, the 2-D FFTs cuFFT's. Options of the
reference that this path does not provide raise ValueError: the
histogram gridding without CIC, normalize=True with its NaN treatments, the
periodic (astropy) convolution, Map_fft without a weight grid, and the
E/B-mode combinations of compute_mcross in the <Map^3> extraction (the cross
maps themselves are available from Map_fft(return_mcross=True)).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import Context, _check, _dp, lib


def _arr(x):
    return np.ascontiguousarray(x, dtype=np.float64)


class _Plan:
    """One tp_apm: grid, field, apertures and filter, with the filters'
    Fourier transforms kept on the device; precision 0 (FP64, the default) or
    1 (FP32 transforms and Fourier products)."""

    def __init__(self, ctx: Context, npix, fieldsize, thetas, polynomial, precision=0):
        self.ctx = ctx
        self.precision = int(precision)
        self.npix = int(npix)
        self.fieldsize = float(fieldsize)
        self.thetas = [float(t) for t in thetas]
        self.polynomial = bool(polynomial)
        self._h = C.c_void_p(0)
        th = _arr(self.thetas)
        _check(ctx._h, lib().tp_apm_create(ctx._h, self.npix, self.fieldsize, _dp(th), len(th), int(polynomial),
                                           self.precision, C.byref(self._h)))
        ctx._adopt(self)

    def close(self):
        if self._h:
            lib().tp_apm_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self, x, y, g):
        x, y = _arr(x), _arr(y)
        g = np.asarray(g)
        g1, g2 = _arr(g.real), _arr(g.imag)
        _check(self.ctx._h, lib().tp_apm_grid(self._h, _dp(x), _dp(y), _dp(g1), _dp(g2), len(x)))

    def get_grid(self):
        n = self.npix
        re, im, w = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
        _check(self.ctx._h, lib().tp_apm_get_grid(self._h, _dp(re), _dp(im), _dp(w)))
        return re + 1j * im, w

    def set_grid(self, shears, weight):
        shears = np.asarray(shears)
        re, im, w = _arr(shears.real), _arr(shears.imag), _arr(weight)
        if re.shape != (self.npix, self.npix) or w.shape != (self.npix, self.npix):
            raise ValueError("grids must be npix x npix")
        _check(self.ctx._h, lib().tp_apm_set_grid(self._h, _dp(re), _dp(im), _dp(w)))

    def maps(self, cross=False):
        n, t = self.npix, len(self.thetas)
        m = np.zeros((t, n, n))
        x = np.zeros((t, n, n)) if cross else None
        _check(self.ctx._h, lib().tp_apm_maps(self._h, _dp(m), _dp(x) if cross else None))
        return (m, x) if cross else m

    def maps_from_kappa(self, kappa):
        n, t = self.npix, len(self.thetas)
        k = _arr(kappa)
        if k.shape != (n, n):
            raise ValueError("kappa must be npix x npix")
        m = np.zeros((t, n, n))
        _check(self.ctx._h, lib().tp_apm_maps_from_kappa(self._h, _dp(k), _dp(m)))
        return m

    def map3(self, same_fieldsize=False):
        t = len(self.thetas)
        out = np.zeros(t * (t + 1) * (t + 2) // 6)
        _check(self.ctx._h, lib().tp_apm_map3(self._h, int(same_fieldsize), _dp(out)))
        return out

    def extract_map3(self, x, y, g, same_fieldsize=True):
        x, y = _arr(x), _arr(y)
        g = np.asarray(g)
        g1, g2 = _arr(g.real), _arr(g.imag)
        t = len(self.thetas)
        out = np.zeros(t * (t + 1) * (t + 2) // 6)
        _check(self.ctx._h, lib().tp_apm_extract_map3(self._h, _dp(x), _dp(y), _dp(g1), _dp(g2), len(x),
                                                      int(same_fieldsize), _dp(out)))
        return out


_shared_ctx = None


def _context(ctx):
    global _shared_ctx
    if ctx is not None:
        return ctx
    if _shared_ctx is None:
        _shared_ctx = Context(0)
    return _shared_ctx


class aperture_mass_computer:
    """The reference class (aperture_mass_computer.py:19-372) on the GPU:
    npix pixels per side, aperture radius theta_ap and field side fieldsize
    in arcmin, exponential filter unless use_polynomial_filter."""

    def __init__(self, npix, theta_ap, fieldsize, use_polynomial_filter=False, ctx: Context | None = None):
        self.npix = int(npix)
        self.theta_ap = float(theta_ap)
        self.fieldsize = float(fieldsize)
        self.use_polynomial_filter = bool(use_polynomial_filter)
        self.ctx = _context(ctx)
        self._plan = None

    def change_theta_ap(self, theta_ap):
        self.theta_ap = float(theta_ap)
        if self._plan is not None:
            self._plan.close()
        self._plan = None

    def _p(self):
        if self._plan is None:
            self._plan = _Plan(self.ctx, self.npix, self.fieldsize, [self.theta_ap], self.use_polynomial_filter)
        return self._plan

    def normalize_shear(self, Xs, Ys, shears, CIC=True, normalize=False, nan_treatment=None, fill_value=0,
                        debug=False):
        if not CIC or normalize or nan_treatment is not None:
            raise ValueError("only the cloud-in-cell gridding without normalisation (CIC=True, normalize=False) "
                             "is provided")
        p = self._p()
        p.grid(Xs, Ys, shears)
        return p.get_grid()

    def Map_fft(self, gamma_arr, norm=None, return_mcross=False, normalize_weighted=True, periodic_boundary=False):
        if norm is None or not normalize_weighted or periodic_boundary:
            raise ValueError("Map_fft needs a weight grid (norm), normalize_weighted=True and zero padding "
                             "(periodic_boundary=False)")
        p = self._p()
        p.set_grid(gamma_arr, norm)
        if return_mcross:
            m, x = p.maps(cross=True)
            return m[0], x[0]
        return p.maps()[0]

    def Map_fft_from_kappa(self, kappa_arr):
        if self.use_polynomial_filter:
            raise ValueError("the U filter of Map_fft_from_kappa is the exponential one")
        return self._p().maps_from_kappa(kappa_arr)[0]


def extract_Map3_of_field(shears, npix, thetas, fieldsize, norm=None, ac=None, compute_mcross=False, save_map=None,
                          same_fieldsize_for_all_theta=False, use_polynomial_filter=False, ctx: Context | None = None):
    """<Map^3> of every triplet of thetas from a shear grid and its weight grid
    (aperture_mass_computer.py:407-531); returns the n(n+1)(n+2)/6 values in the
    reference's loop order."""
    if compute_mcross:
        raise ValueError("compute_mcross (E/B-mode combinations) is not provided")
    if norm is None:
        raise ValueError("a weight grid (norm) is required")
    plan = _Plan(_context(ctx), npix, fieldsize, thetas, use_polynomial_filter)
    try:
        plan.set_grid(shears, norm)
        m = plan.maps()
        if save_map is not None:
            np.save(save_map, np.moveaxis(m, 0, -1))
        return plan.map3(same_fieldsize_for_all_theta)
    finally:
        plan.close()


def extract_Map3(Xs, Ys, shear_catalogue, npix, thetas, fieldsize, compute_mcross=False, save_map=None,
                 same_fieldsize_for_all_theta=True, use_polynomial_filter=False, ctx: Context | None = None):
    """<Map^3> from a shear catalogue (aperture_mass_computer.py:375-405): CIC
    gridding, weighted maps, triplet means, in one device pipeline."""
    if compute_mcross:
        raise ValueError("compute_mcross (E/B-mode combinations) is not provided")
    plan = _Plan(_context(ctx), npix, fieldsize, thetas, use_polynomial_filter)
    try:
        if save_map is not None:
            plan.grid(Xs, Ys, shear_catalogue)
            m = plan.maps()
            np.save(save_map, np.moveaxis(m, 0, -1))
            return plan.map3(same_fieldsize_for_all_theta)
        return plan.extract_map3(Xs, Ys, shear_catalogue, same_fieldsize_for_all_theta)
    finally:
        plan.close()
