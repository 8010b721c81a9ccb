"""threepoint_gb300: GB300 (sm_103a) implementation of threepoint's model path.

Python binding of the C ABI in ``include/threepoint_gb300.h`` (the library
``threepoint_gb300/build/libthreepoint_gb300.so``), with the reference's API
names: ``cosmology``, ``read_n_of_z``, ``read_thetas``,
``convert_angle_to_rad``, ``set_cosmology``, ``MapMapMap``, ``gamma0..3``,
``T1_total``/``T2_total``/``T4_total``.

There is no CPU fallback: every numerical call runs the CUDA kernels of the
shared library, and importing the numerical API without the built library
raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, fields

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libthreepoint_gb300.so")

TP_OK, TP_ERR_ARG, TP_ERR_IO, TP_ERR_FORMAT, TP_ERR_CUDA, TP_ERR_STATE, TP_ERR_CAPACITY, TP_ERR_NOMEM = range(8)
FP64, FP32 = 0, 1
GEOM_CIRCLE, GEOM_SQUARE, GEOM_INFINITE, GEOM_RECTANGLE = 0, 1, 2, 3
N_REDSHIFT_BINS = 256
ARCMIN = 2.9088820866e-4


class ThreepointError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"status {status}: {msg}")
        self.status = status


class _Cosmo(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")]


@dataclass
class cosmology:
    """Cosmological parameters (cuda_version/cosmology.cuh:13-29)."""
    h: float = 0.7
    sigma8: float = 0.8
    omb: float = 0.048
    omc: float = 0.252
    ns: float = 0.96
    w: float = -1.0
    om: float = 0.3
    ow: float = 0.7
    zmax: float = 3.0

    @classmethod
    def flat(cls, om, sigma8, h, w, ns, omb=0.048, zmax=3.0):
        return cls(h=h, sigma8=sigma8, omb=omb, omc=om - omb, ns=ns, w=w, om=om, ow=1 - om, zmax=zmax)

    @classmethod
    def from_file(cls, path):
        c = _Cosmo()
        _check(None, lib().tp_cosmology_from_file(path.encode(), C.byref(c)))
        return cls(**{f.name: getattr(c, f.name) for f in fields(cls)})

    def _c(self):
        return _Cosmo(**{f.name: float(getattr(self, f.name)) for f in fields(self)})


class _CovParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("theta_max", "theta_max_smaller", "shapenoise_sigma", "galaxy_density",
                                           "area")] + [("shapenoise_only", C.c_int)]


@dataclass
class covarianceParameters:
    """Survey parameters of the covariance (cuda_version/cosmology.cuh:44-56);
    angles in rad, galaxy density in rad^-2, area in rad^2."""
    theta_max: float = 0.0
    theta_max_smaller: float = 0.0
    shapenoise_sigma: float = 0.0
    galaxy_density: float = 1.0
    area: float = 0.0
    shapenoise_only: bool = False

    @classmethod
    def from_file(cls, path):
        """cuda_version/cosmology.cu:92-170"""
        c = _CovParams()
        _check(None, lib().tp_cov_params_from_file(str(path).encode(), C.byref(c)))
        return cls(c.theta_max, c.theta_max_smaller, c.shapenoise_sigma, c.galaxy_density, c.area,
                   bool(c.shapenoise_only))


class _GammaConfig(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("rsteps", "usteps", "vsteps")] + [
        (n, C.c_double) for n in ("umin", "umax", "vmin", "vmax", "rmin", "rmax")]


@dataclass
class configGamma:
    """(r, u, v) binning of the shear 3PCF (cuda_version/helpers.cuh:48-52), r in arcmin."""
    rsteps: int = 10
    usteps: int = 10
    vsteps: int = 10
    umin: float = 0.0
    umax: float = 1.0
    vmin: float = -1.0
    vmax: float = 1.0
    rmin: float = 0.1
    rmax: float = 100.0

    @classmethod
    def from_file(cls, path):
        """read_gamma_config (cuda_version/helpers.cu:242-318)"""
        c = _GammaConfig()
        _check(None, lib().tp_gamma_config_from_file(str(path).encode(), C.byref(c)))
        return cls(**{f.name: getattr(c, f.name) for f in fields(cls)})

    def triangles(self):
        """Bin-centre triangles of calculateGamma (calculateGamma.cu:104-121):
        returns x [n,3] (r1, r2, r3) in rad and ruv [n,3] (r [arcmin], u, v)."""
        c = _GammaConfig(**{f.name: getattr(self, f.name) for f in fields(self)})
        n = self.rsteps * self.usteps * self.vsteps
        x, ruv = np.zeros(3 * n), np.zeros(3 * n)
        _check(None, lib().tp_gamma_triangles(C.byref(c), _dp(x), _dp(ruv)))
        return x.reshape(n, 3), ruv.reshape(n, 3)


_lib = None


def lib():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run threepoint_gb300.build.build() or __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        d, i, p, l = C.c_double, C.c_int, C.c_void_p, C.c_long
        dp, ip, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64)
        L.tp_status_string.restype = C.c_char_p
        L.tp_status_string.argtypes = [i]
        L.tp_last_error.restype = C.c_char_p
        L.tp_last_error.argtypes = [p]
        L.tp_version.restype = C.c_char_p
        L.tp_cosmology_from_file.argtypes = [C.c_char_p, C.POINTER(_Cosmo)]
        L.tp_read_n_of_z.argtypes = [C.c_char_p, i, d, dp]
        L.tp_rebin_n_of_z.argtypes = [dp, dp, i, i, d, dp]
        L.tp_read_thetas.argtypes = [C.c_char_p, dp, i, ip]
        L.tp_convert_angle_to_rad.argtypes = [d, C.c_char_p, dp]
        L.tp_ctx_create.argtypes = [i, C.POINTER(p)]
        L.tp_ctx_destroy.argtypes = [p]
        L.tp_set_cosmologies.argtypes = [p, C.POINTER(_Cosmo), i, dp, i, dp, d, d, d]
        L.tp_set_shape_noise.argtypes = [p, d, d, i]
        L.tp_get_tables.argtypes = [p, i, dp]
        L.tp_bkappa_batch.argtypes = [p, ip, dp, l, i, dp]
        L.tp_pell_batch.argtypes = [p, i, dp, l, i, dp]
        L.tp_bkappa_nodes.argtypes = [p, i, dp, l, i, dp, dp]
        L.tp_gamma_integrand_points.argtypes = [p, i, dp, i, dp, i, i, dp]
        L.tp_apm_create.argtypes = [p, i, d, dp, i, i, i, C.POINTER(p)]
        L.tp_apm_destroy.argtypes = [p]
        L.tp_apm_fft_size.argtypes = [p]
        L.tp_apm_grid.argtypes = [p, dp, dp, dp, dp, l]
        L.tp_apm_grid_device.argtypes = [p, p, p, p, p, l]
        L.tp_apm_set_grid.argtypes = [p, dp, dp, dp]
        L.tp_apm_get_grid.argtypes = [p, dp, dp, dp]
        L.tp_apm_maps.argtypes = [p, dp, dp]
        L.tp_apm_maps_from_kappa.argtypes = [p, dp, dp]
        L.tp_apm_map3.argtypes = [p, i, dp]
        L.tp_apm_extract_map3.argtypes = [p, dp, dp, dp, dp, l, i, dp]
        L.tp_apm_extract_map3_device.argtypes = [p, p, p, p, p, l, i, p]
        L.tp_map3_batch.argtypes = [p, ip, i, dp, i, d, d, d, d, d, i, dp, dp, i64p, ip]
        L.tp_map3_jobs_device.argtypes = [p, p, p, i, d, d, d, d, d, i, p, p, p, p, p, p]
        L.tp_ctx_set_limits.argtypes = [p, i, i]
        L.tp_ctx_set_escalation.argtypes = [p, i]
        L.tp_map3_jobs_noalloc.argtypes = [p, p, p, i, d, d, d, d, d, i, p, p, p]
        L.tp_ctx_stream.restype = p
        L.tp_ctx_stream.argtypes = [p]
        L.tp_pipe_peaks.argtypes = [i, dp]
        L.tp_gamma_batch.argtypes = [p, i, dp, i, i, d, i, dp, ip]
        L.tp_ogata_weights.argtypes = [dp]
        L.tp_cov_total_batch.argtypes = [p, i, i, i, d, d, dp, dp, i, i, dp, ip]
        L.tp_cov_term_batch.argtypes = [p, i, i, i, d, d, dp, i, i, dp, ip]
        L.tp_set_rectangle_side.argtypes = [p, d]
        L.tp_halo_tables.argtypes = [p, i, dp]
        L.tp_halo_los.argtypes = [p, i, dp, l, i, dp, dp]
        L.tp_halo_integrand_points.argtypes = [p, i, i, i, d, dp, dp, l, i, dp]
        L.tp_ctx_set_cov_tolerance.argtypes = [p, i, d]
        L.tp_ctx_set_halo_cluster.argtypes = [p, i]
        L.tp_ctx_set_map3_cluster.argtypes = [p, i]
        L.tp_cov_params_from_file.argtypes = [C.c_char_p, C.POINTER(_CovParams)]
        L.tp_gamma_config_from_file.argtypes = [C.c_char_p, C.POINTER(_GammaConfig)]
        L.tp_gamma_triangles.argtypes = [C.POINTER(_GammaConfig), dp, dp]
        L.tp_likelihood_create.argtypes = [i, dp, dp, i, C.POINTER(p)]
        L.tp_likelihood_destroy.argtypes = [p]
        L.tp_likelihood_destroy.restype = None
        L.tp_likelihood_last_error.argtypes = [p]
        L.tp_likelihood_last_error.restype = C.c_char_p
        L.tp_likelihood_cov_inv.argtypes = [p, dp]
        L.tp_likelihood_chi2.argtypes = [p, dp, i, dp]
        L.tp_likelihood_chi2_device.argtypes = [p, p, i, l, p, p]
        L.tp_mlp_param_count.restype = l
        L.tp_mlp_param_count.argtypes = []
        L.tp_mlp_create.argtypes = [i, i, C.POINTER(p)]
        L.tp_mlp_destroy.argtypes = [p]
        L.tp_mlp_destroy.restype = None
        L.tp_mlp_last_error.argtypes = [p]
        L.tp_mlp_last_error.restype = C.c_char_p
        L.tp_mlp_set_params.argtypes = [p, dp]
        L.tp_mlp_get_params.argtypes = [p, dp]
        L.tp_mlp_forward.argtypes = [p, dp, l, dp]
        L.tp_mlp_gradients.argtypes = [p, dp, dp, l, dp, dp]
        L.tp_mlp_train_step_device.argtypes = [p, p, p, l, C.c_float, p]
        L.tp_mlp_sync.argtypes = [p]
        L.tp_mlp_stream.argtypes = [p]
        L.tp_mlp_stream.restype = p
        L.tp_gemm_bf16_device.argtypes = [p, p, i, p, i, p, i, i, i, i]
        _lib = L
    return _lib


def _check(ctx, st):
    if st != TP_OK:
        L = lib()
        msg = L.tp_status_string(st).decode()
        if ctx is not None:
            detail = L.tp_last_error(ctx).decode()
            if detail:
                msg += ": " + detail
        raise ThreepointError(st, msg)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _arr(x, dtype=np.float64):
    return np.ascontiguousarray(x, dtype=dtype)


# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def read_n_of_z(path, n_bins=N_REDSHIFT_BINS, zmax=3.0):
    """cuda_version/helpers.cu:9-128"""
    out = np.zeros(n_bins)
    _check(None, lib().tp_read_n_of_z(str(path).encode(), n_bins, zmax, _dp(out)))
    return out


def rebin_n_of_z(zs, ns, n_bins=N_REDSHIFT_BINS, zmax=3.0):
    """read_n_of_z's rebinning of an in-memory (z, n) table (helpers.cu:37-128)"""
    zs, ns = _arr(zs), _arr(ns)
    out = np.zeros(n_bins)
    _check(None, lib().tp_rebin_n_of_z(_dp(zs), _dp(ns), len(zs), n_bins, zmax, _dp(out)))
    return out


def read_thetas(path, cap=4096):
    """cuda_version/helpers.cu:176-200"""
    out = np.zeros(cap)
    n = C.c_int(0)
    _check(None, lib().tp_read_thetas(str(path).encode(), _dp(out), cap, C.byref(n)))
    return out[: min(n.value, cap)].copy()


def convert_angle_to_rad(value, unit="arcmin"):
    """cuda_version/helpers.cu:130-153"""
    out = C.c_double(0)
    _check(None, lib().tp_convert_angle_to_rad(float(value), unit.encode(), C.byref(out)))
    return out.value


def theta_triplets(thetas):
    """theta1<=theta2<=theta3 combinations in the reference's loop order
    (cuda_version/calculateApertureStatistics.cu:92-115)."""
    n = len(thetas)
    return [(thetas[i], thetas[j], thetas[k]) for i in range(n) for j in range(i, n) for k in range(j, n)]


# ---------------------------------------------------------------------------
class Context:
    """One CUDA device + stream + the device tables of a batch of cosmologies."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p(0)
        _check(None, lib().tp_ctx_create(device, C.byref(self._h)))
        self.n_cosmo = 0
        self.cosmologies = []

    def set_limits(self, region_cap=32768, max_ctas=0):
        """Regions per adaptive integral and CTAs of the persistent grid."""
        _check(self._h, lib().tp_ctx_set_limits(self._h, region_cap, max_ctas))

    def _adopt(self, child):
        """Objects holding device state made with this context (aperture-mass
        plans) are closed before the context."""
        import weakref

        if not hasattr(self, "_children"):
            self._children = []
        self._children.append(weakref.ref(child))

    def set_escalation(self, max_region_cap=1 << 24):
        """Integrals of map3_batch / gamma_batch that reach the region cap are
        integrated again with larger caps up to max_region_cap (0: off)."""
        _check(self._h, lib().tp_ctx_set_escalation(self._h, max_region_cap))

    def close(self):
        for r in getattr(self, "_children", []):
            c = r()
            if c is not None:
                c.close()
        self._children = []
        if self._h:
            lib().tp_ctx_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- set_cosmology (cuda_version/bispectrum.cu:100-219), batched --------
    def set_cosmologies(self, cosmos, nz, pk=None, dk=0.0, kmin=0.0, kmax=0.0):
        cosmos = list(cosmos)
        arr = (_Cosmo * len(cosmos))(*[c._c() for c in cosmos])
        nz = _arr(nz)
        stride = 0 if nz.ndim == 1 else N_REDSHIFT_BINS
        if nz.size not in (N_REDSHIFT_BINS, N_REDSHIFT_BINS * len(cosmos)):
            raise ValueError("nz must hold 256 values or 256 per cosmology")
        pkp = None
        if pk is not None:
            pk = _arr(pk)
            if pk.size != 256 * len(cosmos):
                pk = np.tile(pk.reshape(-1)[:256], len(cosmos))
            pkp = _dp(pk)
        _check(self._h, lib().tp_set_cosmologies(self._h, arr, len(cosmos), _dp(nz), stride, pkp, dk, kmin, kmax))
        self.n_cosmo = len(cosmos)
        self.cosmologies = cosmos

    def set_cosmology(self, cosmo, nz, pk=None, dk=0.0, kmin=0.0, kmax=0.0):
        self.set_cosmologies([cosmo], nz, pk, dk, kmin, kmax)

    def set_shape_noise(self, sigma_eps, n_gal_per_rad2, constant_powerspectrum=False):
        _check(self._h, lib().tp_set_shape_noise(self._h, sigma_eps, n_gal_per_rad2, int(constant_powerspectrum)))

    def set_rectangle_side(self, theta_max_smaller):
        """Second side [rad] of a rectangular survey (GEOM_RECTANGLE)."""
        _check(self._h, lib().tp_set_rectangle_side(self._h, theta_max_smaller))

    def tables(self, i=0):
        out = np.zeros(6 * 256 + 1)
        _check(self._h, lib().tp_get_tables(self._h, i, _dp(out)))
        names = ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur")
        d = {n: out[k * 256:(k + 1) * 256].copy() for k, n in enumerate(names)}
        d["norm"] = out[-1]
        return d

    # -- point evaluations ---------------------------------------------------
    def bkappa(self, ell, cosmo_index=None, precision=FP64):
        ell = _arr(ell).reshape(-1, 3)
        out = np.zeros(len(ell))
        ip = None
        if cosmo_index is not None:
            ci = _arr(np.broadcast_to(cosmo_index, (len(ell),)), np.int32)
            ip = ci.ctypes.data_as(C.POINTER(C.c_int))
        _check(self._h, lib().tp_bkappa_batch(self._h, ip, _dp(ell), len(ell), precision, _dp(out)))
        return out

    def bkappa_nodes(self, ell, cosmo_index=0, precision=FP64):
        """The 96 line-of-sight terms of bkappa per triangle (they sum to
        bkappa) and the bispectrum at each node: two [n][96] arrays."""
        ell = _arr(ell).reshape(-1, 3)
        term = np.zeros((len(ell), 96))
        bis = np.zeros((len(ell), 96))
        _check(self._h, lib().tp_bkappa_nodes(self._h, cosmo_index, _dp(ell), len(ell), precision, _dp(term),
                                              _dp(bis)))
        return term, bis

    def gamma_integrand_points(self, which, x, pts, cosmo_index=0, precision=FP64):
        """The Gamma^0 (which=0) or Gamma^1 (which=1) cubature integrand of
        triangle x at points (z, phi, psi), summed over the Ogata nodes."""
        x = _arr(x).reshape(3)
        pts = _arr(pts).reshape(-1, 3)
        out = np.zeros(2 * len(pts))
        _check(self._h, lib().tp_gamma_integrand_points(self._h, cosmo_index, _dp(x), which, _dp(pts), len(pts),
                                                        precision, _dp(out)))
        return out[0::2] + 1j * out[1::2]

    def Pell(self, ell, cosmo_index=0, precision=FP64):
        ell = _arr(ell).reshape(-1)
        out = np.zeros(len(ell))
        _check(self._h, lib().tp_pell_batch(self._h, cosmo_index, _dp(ell), len(ell), precision, _dp(out)))
        return out

    # -- <Map^3> (cuda_version/apertureStatistics.cu:201-230) -------------
    def map3_batch(self, thetas, cosmo_index=None, phiMin=0.0, phiMax=2 * math.pi, lMin=1.0, lMax=0.0,
                   rel_tol=1e-4, precision=FP64, return_info=False, check=True):
        th = _arr(thetas).reshape(-1, 3)
        if cosmo_index is None:
            cosmo_index = list(range(self.n_cosmo))
        ci = _arr(cosmo_index, np.int32).reshape(-1)
        nc, nt = len(ci), len(th)
        out = np.zeros(nc * nt)
        err = np.zeros(nc * nt)
        nev = np.zeros(nc * nt, dtype=np.int64)
        st = np.zeros(nc * nt, dtype=np.int32)
        rc = lib().tp_map3_batch(self._h, ci.ctypes.data_as(C.POINTER(C.c_int)), nc, _dp(th), nt, phiMin, phiMax,
                                 lMin, lMax, rel_tol, precision, _dp(out), _dp(err),
                                 nev.ctypes.data_as(C.POINTER(C.c_int64)), st.ctypes.data_as(C.POINTER(C.c_int)))
        if check or rc != TP_ERR_CAPACITY:
            _check(self._h, rc)
        out, err, nev, st = (a.reshape(nc, nt) for a in (out, err, nev, st))
        if return_info:
            return out, dict(err=err, neval=nev, status=st)
        return out

    def MapMapMap(self, thetas, phiMin=0.0, phiMax=2 * math.pi, lMin=1.0, precision=FP64, cosmo_index=0):
        """<Map^3>(theta1, theta2, theta3) [rad] of one cosmology
        (apertureStatistics.cuh:106)."""
        return float(self.map3_batch([thetas], [cosmo_index], phiMin, phiMax, lMin, precision=precision)[0, 0])

    def map3_jobs_device(self, job_cosmo, job_theta, out, err=None, neval=None, status=None, phiMin=0.0,
                         phiMax=2 * math.pi, lMin=1.0, lMax=0.0, rel_tol=1e-4, precision=FP32, nlive=None,
                         job_order=None):
        """Asynchronous device-resident variant: arguments are torch CUDA
        tensors (int32 [n], float64 [n,3], float64 [n] ...)."""
        n = int(job_cosmo.numel())
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
        _check(self._h, lib().tp_map3_jobs_device(self._h, ptr(job_cosmo), ptr(job_theta), n, phiMin, phiMax, lMin,
                                                  lMax, rel_tol, precision, ptr(out), ptr(err), ptr(neval),
                                                  ptr(nlive), ptr(status), ptr(job_order)))

    @property
    def stream_handle(self):
        """The library stream of this context (an int cudaStream_t)."""
        return lib().tp_ctx_stream(self._h)

    # -- shear 3PCF (cuda_version/gamma.cu:98-148) ---------------------------
    def gamma_batch(self, x, comp_mask=0xF, rel_tol=1e-3, precision=FP64, cosmo_index=0, check=True):
        """With check=False, triangles whose integrals hit a region or sweep
        cap do not raise; their per-triangle status is left in
        self.last_gamma_status (0 = converged)."""
        x = _arr(x).reshape(-1, 3)
        out = np.zeros(len(x) * 8)
        st = np.zeros(len(x), dtype=np.int32)
        rc = lib().tp_gamma_batch(self._h, cosmo_index, _dp(x), len(x), comp_mask, rel_tol, precision, _dp(out),
                                  st.ctypes.data_as(C.POINTER(C.c_int)))
        self.last_gamma_status = st
        if check or rc != TP_ERR_CAPACITY:
            _check(self._h, rc)
        o = out.reshape(-1, 4, 2)
        return o[..., 0] + 1j * o[..., 1]

    def gamma0(self, x1, x2, x3, **kw):
        return complex(self.gamma_batch([(x1, x2, x3)], comp_mask=1, **kw)[0, 0])

    def gamma1(self, x1, x2, x3, **kw):
        return complex(self.gamma_batch([(x1, x2, x3)], comp_mask=2, **kw)[0, 1])

    def gamma2(self, x1, x2, x3, **kw):
        return complex(self.gamma_batch([(x1, x2, x3)], comp_mask=4, **kw)[0, 2])

    def gamma3(self, x1, x2, x3, **kw):
        return complex(self.gamma_batch([(x1, x2, x3)], comp_mask=8, **kw)[0, 3])

    # -- covariance (cuda_version/apertureStatisticsCovariance.cu:272-683) --
    def cov_total(self, term, th123, th456, geometry=GEOM_SQUARE, thetaMax=0.0, area=0.0, precision=FP64,
                  cosmo_index=0, check=True):
        """T1_total / T2_total / T4_total / T5_total / T6_total / T7_total for
        pairs of triplets (apertureStatisticsCovariance.cu:272-1044). With
        check=False an integral that hit its region or sweep cap does not
        raise; the number of such integrals is left in self.last_capped."""
        a = _arr(th123).reshape(-1, 3)
        b = _arr(th456).reshape(-1, 3)
        out = np.zeros(len(a))
        nb = C.c_int(0)
        rc = lib().tp_cov_total_batch(self._h, cosmo_index, term, geometry, thetaMax, area, _dp(a), _dp(b), len(a),
                                      precision, _dp(out), C.byref(nb))
        self.last_capped = nb.value
        if check or rc != TP_ERR_CAPACITY:
            _check(self._h, rc)
        return out

    def cov_term(self, term, th6, geometry=GEOM_SQUARE, thetaMax=0.0, area=0.0, precision=FP64, cosmo_index=0):
        """Single terms T1/T2/T4/T5/T6/T7(theta1..theta6)
        (apertureStatisticsCovariance.cu:1065-1313)."""
        t = _arr(th6).reshape(-1, 6)
        out = np.zeros(len(t))
        nb = C.c_int(0)
        _check(self._h, lib().tp_cov_term_batch(self._h, cosmo_index, term, geometry, thetaMax, area, _dp(t), len(t),
                                                precision, _dp(out), C.byref(nb)))
        return out

    def T1_total(self, th123, th456, **kw):
        return float(self.cov_total(1, [th123], [th456], **kw)[0])

    def T2_total(self, th123, th456, **kw):
        return float(self.cov_total(2, [th123], [th456], **kw)[0])

    def T4_total(self, th123, th456, **kw):
        return float(self.cov_total(4, [th123], [th456], **kw)[0])

    def T5_total(self, th123, th456, **kw):
        return float(self.cov_total(5, [th123], [th456], **kw)[0])

    def T6_total(self, th123, th456, **kw):
        return float(self.cov_total(6, [th123], [th456], **kw)[0])

    def T7_total(self, th123, th456, **kw):
        return float(self.cov_total(7, [th123], [th456], **kw)[0])

    @staticmethod
    def T7_2h_total(th123, th456, geometry=GEOM_SQUARE, **kw):
        """T7_2h_total (apertureStatisticsCovariance.cu:1046-1063,1315-1356):
        0 for the infinite survey, and 0 for the square because the reference's
        integrand multiplies by a survey-variance table it never fills; the
        reference throws for the circle and the rectangle (ValueError here)."""
        if len(th123) != 3 or len(th456) != 3:
            raise ValueError("T7_2h_total: Wrong number of aperture radii")
        if geometry in (GEOM_SQUARE, GEOM_INFINITE):
            return 0.0
        raise ValueError("T7_SSC: Wrong survey geometry, only coded for square survey")

    # -- halo model (cuda_version/halomodel.cu) --
    def set_cov_tolerance(self, term, rel_tol):
        """Relative tolerance of the T5/T6/T7 integrals (0 = the reference's
        1e-2 / 1e-1 / 1e-1)."""
        _check(self._h, lib().tp_ctx_set_cov_tolerance(self._h, term, rel_tol))

    def set_map3_cluster(self, on=True):
        """<Map^3> batches with no more integrals than CTA slots: one 8-CTA
        cluster per integral (on) or one CTA (off); 2: clusters for every batch."""
        _check(self._h, lib().tp_ctx_set_map3_cluster(self._h, 2 if on == 2 else int(bool(on))))

    def set_halo_cluster(self, ctas=16):
        """CTAs per T5/T6/T7 integral: 16 (a 16-CTA cluster where the batch
        leaves room, else 8), 8 (8-CTA clusters) or 1."""
        _check(self._h, lib().tp_ctx_set_halo_cluster(self._h, ctas))

    def halo_tables(self, cosmo_index=0):
        """(sigma^2(m_i), dsigma^2/dm(m_i)) at z = 0, 128 masses each."""
        out = np.zeros(256)
        _check(self._h, lib().tp_halo_tables(self._h, cosmo_index, _dp(out)))
        return out[:128].copy(), out[128:].copy()

    def halo_los(self, pts, cosmo_index=0, precision=FP64):
        """One-halo line-of-sight trispectrum (l1..l4) and pentaspectrum
        (l1..l6) at rows (m, l1, ..., l6)."""
        pts = _arr(pts).reshape(-1, 7)
        tri, pen = np.zeros(len(pts)), np.zeros(len(pts))
        _check(self._h, lib().tp_halo_los(self._h, cosmo_index, _dp(pts), len(pts), precision, _dp(tri), _dp(pen)))
        return tri, pen

    def halo_integrand(self, term, th6, x, geometry=GEOM_INFINITE, thetaMax=0.0, cosmo_index=0, precision=FP64):
        """Integrand of T5 (rows of 6) / T6, T7 (rows of 7) at points x, before
        the 1/area/(2 pi)^n normalisation."""
        nd = 6 if term == 5 else 7
        x = _arr(x).reshape(-1, nd)
        th = _arr(th6)
        out = np.zeros(len(x))
        _check(self._h, lib().tp_halo_integrand_points(self._h, cosmo_index, term, geometry, thetaMax, _dp(th),
                                                        _dp(x), len(x), precision, _dp(out)))
        return out


class Likelihood:
    """Gaussian likelihood of <Map^3> model vectors against a measurement
    (cosmosis/threepoint_likelihood.py:8-58): chi2 = (m-d)^T C^-1 (m-d),
    log L = -chi2/2. The covariance is factored once on the GPU."""

    def __init__(self, data, cov, device=0):
        d = _arr(data).reshape(-1)
        c = _arr(cov).reshape(len(d), len(d))
        self.n = len(d)
        self._h = C.c_void_p(0)
        st = lib().tp_likelihood_create(device, _dp(d), _dp(c), self.n, C.byref(self._h))
        if st == TP_ERR_ARG:
            raise ThreepointError(st, "covariance is not positive definite (or has non-finite entries)")
        _check(None, st)

    def cov_inv(self):
        out = np.zeros((self.n, self.n))
        self._chk(lib().tp_likelihood_cov_inv(self._h, _dp(out)))
        return out

    def chi2(self, models):
        m = _arr(models).reshape(-1, self.n)
        out = np.zeros(len(m))
        self._chk(lib().tp_likelihood_chi2(self._h, _dp(m), len(m), _dp(out)))
        return out

    def loglike(self, models):
        return -0.5 * self.chi2(models)

    def chi2_device(self, models, out, stream=None):
        """models: CUDA float64 tensor [B, >=n] (row stride >= n); out: [B]."""
        self._chk(lib().tp_likelihood_chi2_device(self._h, C.c_void_p(models.data_ptr()), int(models.shape[0]),
                                                  int(models.stride(0)), C.c_void_p(out.data_ptr()),
                                                  C.c_void_p(stream) if stream else None))

    def _chk(self, st):
        if st != TP_OK:
            raise ThreepointError(st, lib().tp_likelihood_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib().tp_likelihood_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """The b_kappa surrogate network (8 -> 256 x 4 -> 1, SiLU) on the tensor
    cores: BF16 operands, FP32 accumulation and master parameters, Adam.

    Parameters are a list [(W [out, in], b [out])] of five layers, or the flat
    FP64 array of the C ABI (tp_mlp_param_count() values)."""

    WIDTHS = (8, 256, 256, 256, 256, 1)

    def __init__(self, max_batch=65536, device=0):
        self._h = C.c_void_p(0)
        self.device = device
        self.max_batch = max_batch
        st = lib().tp_mlp_create(device, max_batch, C.byref(self._h))
        if st != TP_OK:
            self._h = C.c_void_p(0)
            raise ThreepointError(st, f"tp_mlp_create(device={device}, max_batch={max_batch}) failed")

    @staticmethod
    def param_count():
        return int(lib().tp_mlp_param_count())

    @classmethod
    def flatten(cls, params):
        return np.concatenate([np.concatenate([np.asarray(W, dtype=np.float64).reshape(-1),
                                               np.asarray(b, dtype=np.float64).reshape(-1)]) for W, b in params])

    @classmethod
    def unflatten(cls, flat):
        out, o = [], 0
        for i in range(len(cls.WIDTHS) - 1):
            fi, fo = cls.WIDTHS[i], cls.WIDTHS[i + 1]
            W = flat[o:o + fi * fo].reshape(fo, fi)
            o += fi * fo
            out.append((W, flat[o:o + fo].copy()))
            o += fo
        return out

    def set_params(self, params):
        flat = params if isinstance(params, np.ndarray) and params.ndim == 1 else self.flatten(params)
        flat = _arr(flat)
        if flat.size != self.param_count():
            raise ValueError(f"{flat.size} parameters for {self.param_count()}")
        self._chk(lib().tp_mlp_set_params(self._h, _dp(flat)))

    def get_params(self, flat=False):
        out = np.zeros(self.param_count())
        self._chk(lib().tp_mlp_get_params(self._h, _dp(out)))
        return out if flat else self.unflatten(out)

    def forward(self, x):
        x = _arr(x).reshape(-1, 8)
        y = np.zeros(len(x))
        self._chk(lib().tp_mlp_forward(self._h, _dp(x), len(x), _dp(y)))
        return y

    def gradients(self, x, t):
        """(loss, [(dW, db)]) of the mean squared error on one batch"""
        x = _arr(x).reshape(-1, 8)
        t = _arr(t).reshape(-1)
        g = np.zeros(self.param_count())
        loss = C.c_double(0)
        self._chk(lib().tp_mlp_gradients(self._h, _dp(x), _dp(t), len(x), _dp(g), C.byref(loss)))
        return loss.value, self.unflatten(g)

    def train_step_device(self, x, t, lr, loss_out=None):
        """x: CUDA float32 [n, 8], t: [n]; asynchronous on self.stream_handle"""
        self._chk(lib().tp_mlp_train_step_device(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                                 int(t.numel()), float(lr),
                                                 C.c_void_p(loss_out.data_ptr()) if loss_out is not None else None))

    def sync(self):
        self._chk(lib().tp_mlp_sync(self._h))

    @property
    def stream_handle(self):
        return lib().tp_mlp_stream(self._h)

    def gemm_device(self, A, B, Cout):
        """Cout = A B^T on the tensor cores (torch CUDA tensors: A, B bfloat16
        [M, K], [N, K] row-major; Cout float32 [M, N])"""
        M, K = A.shape
        N = B.shape[0]
        self._chk(lib().tp_gemm_bf16_device(self._h, C.c_void_p(A.data_ptr()), int(A.stride(0)),
                                            C.c_void_p(B.data_ptr()), int(B.stride(0)), C.c_void_p(Cout.data_ptr()),
                                            int(Cout.stride(0)), int(M), int(N), int(K)))

    def _chk(self, st):
        if st != TP_OK:
            raise ThreepointError(st, lib().tp_mlp_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib().tp_mlp_destroy(self._h)
            self._h = C.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ogata_weights():
    out = np.zeros(4 * 33)
    _check(None, lib().tp_ogata_weights(_dp(out)))
    return out.reshape(4, 33)


def version():
    return lib().tp_version().decode()


def pipe_peaks(device=0):
    """Measured whole-device throughput: (SFU ex2 ops/s, FP32 FMA/s, FP64 FMA/s)."""
    out = np.zeros(3)
    _check(None, lib().tp_pipe_peaks(device, _dp(out)))
    return tuple(out)
