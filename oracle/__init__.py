"""CPU FP64 oracle for the threepoint model-evaluation path.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` leg of ``bench.py``. It is the checker; the product
(package ``threepoint_gb300``) never imports it.

The numerics live in ``oracle.cpp`` (a C++ FP64 restatement of the reference's
cuda_version semantics, built into ``oracle/build/liboracle.so``). This module
holds the ctypes binding plus pure-Python restatements of the small input
helpers (``read_n_of_z``, the ``.param`` reader, theta-triplet enumeration).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_host.so")

NZ = 256
ARCMIN = 2.9088820866e-4  # convert_angle_to_rad, cuda_version/helpers.cu:137


class Cosmo(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")]


class CovParams(C.Structure):
    _fields_ = [("type", C.c_int), ("thetaMax", C.c_double), ("area", C.c_double), ("lMin", C.c_double),
                ("thetaMaxSmaller", C.c_double)]


INTEGRAND_V = C.CFUNCTYPE(C.c_int, C.c_uint, C.c_size_t, C.POINTER(C.c_double), C.c_void_p, C.c_uint,
                          C.POINTER(C.c_double))


def build(quiet: bool = True) -> str:
    """Compile liboracle.so (make in this directory)."""
    out = subprocess.run(["make", "-C", HERE, "build/liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        d, p, i, l = C.c_double, C.c_void_p, C.c_int, C.c_long
        dp = C.POINTER(C.c_double)
        L.orc_tables_create.restype = p
        L.orc_tables_create.argtypes = [C.POINTER(Cosmo), dp, dp, d, d, d]
        L.orc_tables_destroy.argtypes = [p]
        L.orc_tables_get.argtypes = [p, dp]
        L.orc_set_noise.argtypes = [p, d, d, i]
        L.orc_set_analytic.argtypes = [p, i]
        for name, nargs in (("orc_E", 1), ("orc_linear_pk", 1), ("orc_lgr", 1), ("orc_calc_r_sigma", 1),
                            ("orc_f_K_at_z", 1), ("orc_P_k_nonlinear", 2), ("orc_bispec_at_z", 4),
                            ("orc_integrand_bkappa", 4), ("orc_bkappa", 3), ("orc_Pell", 1), ("orc_limber_integrand", 2)):
            f = getattr(L, name)
            f.restype = d
            f.argtypes = [p] + [d] * nargs
        L.orc_sigmam.restype = d
        L.orc_sigmam.argtypes = [p, d, i]
        L.orc_bkappa_batch.argtypes = [p, dp, l, dp]
        L.orc_uHat.restype = d
        L.orc_uHat.argtypes = [d]
        L.orc_gq96.argtypes = [dp, dp]
        L.orc_hcubature_v.restype = i
        L.orc_hcubature_v.argtypes = [C.c_uint, p, p, C.c_uint, dp, dp, C.c_size_t, d, d, i, dp, dp]
        L.orc_last_neval.restype = l
        L.orc_map3_ctx_create.restype = p
        L.orc_map3_ctx_create.argtypes = [p, d, d, d]
        L.orc_map3_ctx_destroy.argtypes = [p]
        L.orc_MapMapMap.restype = d
        L.orc_MapMapMap.argtypes = [p, dp, d, d, d, d, d, dp, C.POINTER(l)]
        L.orc_ogata_weights.argtypes = [dp]
        L.orc_gamma.argtypes = [p, i, d, d, d, d, d, dp, dp, C.POINTER(l)]
        L.orc_ggg_analytic.argtypes = [d, d, d, dp, dp]
        L.orc_gamma_integrand_points.argtypes = [p, i, d, d, d, dp, l, dp]
        cp = C.POINTER(CovParams)
        L.orc_T1.restype = d
        L.orc_T1.argtypes = [p, cp, dp, d, C.POINTER(l)]
        L.orc_T1_capped.restype = d
        L.orc_T1_capped.argtypes = [p, cp, dp, d, l, dp, C.POINTER(l)]
        L.orc_T2.restype = d
        L.orc_T2.argtypes = [p, cp, dp]
        L.orc_T4.restype = d
        L.orc_T4.argtypes = [p, cp, dp, d, C.POINTER(l)]
        for n in ("orc_T1_total", "orc_T2_total", "orc_T4_total"):
            getattr(L, n).restype = d
            getattr(L, n).argtypes = [p, cp, dp, dp]
        L.orc_G_square.restype = d
        L.orc_G_square.argtypes = [d, d, d]
        L.orc_halo_tables.argtypes = [p, dp]
        L.orc_total_probe.restype = d
        L.orc_total_probe.argtypes = [i, i, p, dp, dp]
        L.orc_halo_ctx_create.restype = p
        L.orc_halo_ctx_create.argtypes = [p, cp, i, dp]
        L.orc_halo_ctx_destroy.argtypes = [p]
        L.orc_halo_ctx_lmax.restype = d
        L.orc_halo_ctx_lmax.argtypes = [p]
        for n, k in (("orc_hmf", 2), ("orc_u_nfw", 3), ("orc_get_sigma2", 2), ("orc_get_dsigma2", 2),
                     ("orc_r_200", 1)):
            getattr(L, n).restype = d
            getattr(L, n).argtypes = [p] + [d] * k
        L.orc_concentration.restype = d
        L.orc_concentration.argtypes = [d, d]
        L.orc_sici.argtypes = [d, dp, dp]
        L.orc_halo_los.argtypes = [p, dp, l, dp, dp]
        L.orc_halo_integrand.argtypes = [p, cp, i, dp, d, dp, l, dp]
        L.orc_T_halo.restype = d
        L.orc_T_halo.argtypes = [p, cp, i, dp, d, l, dp, C.POINTER(l)]
        L.orc_halo_total_terms.restype = i
        L.orc_halo_total_terms.argtypes = [i, dp, dp, C.POINTER(i), C.POINTER(i)]
        L.orc_T_halo_total.restype = d
        L.orc_T_halo_total.argtypes = [p, cp, i, dp, dp, d, l]
        L.orc_set_threads.argtypes = [i]
        _lib = L
    return _lib


def _dp(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


# ---------------------------------------------------------------------------
# input helpers (pure-Python restatements)
# ---------------------------------------------------------------------------
def read_param_file(path: str) -> dict:
    """``.param`` reader: ``name value`` lines, '#' comments
    (cuda_version/cosmology.cu:11-78). Returns the cosmology dict with
    ow = 1 - om and omc = om - omb."""
    vals = {}
    keymap = {"h": "h", "sigma_8": "sigma8", "Omega_b": "omb", "n_s": "ns", "w": "w", "Omega_m": "om",
              "z_max": "zmax"}
    with open(path) as f:
        for line in f:
            if not line.strip() or line.startswith("#"):
                continue
            parts = line.split()
            if parts[0] not in keymap:
                break
            vals[keymap[parts[0]]] = float(parts[1])
    vals["ow"] = 1 - vals["om"]
    vals["omc"] = vals["om"] - vals["omb"]
    return vals


def read_n_of_z(zs, ns, n_bins: int, zmax: float) -> np.ndarray:
    """Rebin a tabulated n(z) to ``n_bins`` bins at i*dz and normalise
    sum(n)*dz = 1 (cuda_version/helpers.cu:9-128)."""
    zs = [float(z) for z in zs]
    ns = [float(n) for n in ns]
    nf = len(zs)
    zmin_f, zmax_f = zs[0], zs[-1]
    dz_f = (zmax_f - zmin_f) / (nf - 1)
    dz = zmax / n_bins
    out = []
    if dz > dz_f:
        for i in range(n_bins):
            z = i * dz
            ix = int((z - zmin_f) / dz_f)
            dix = (z - zmin_f) / dz_f - ix
            v = 0.0
            if 0 <= ix < nf - 1:
                v = ns[ix + 1] * dix + ns[ix] * (1 - dix)
            if ix >= nf - 1:
                v = 0.0
            out.append(v)
    else:
        for i in range(n_bins):
            z_low, z_up = i * dz, (i + 1) * dz
            k = l = 0
            for j in range(nf):
                if zs[j] < z_low:
                    k = j
                if zs[j] < z_up:
                    l = j
            v = 0.0
            if z_up < zmin_f or k > nf:
                v = 0.0
            elif l - k <= 1:
                if k == l:
                    v = ns[k]
                elif l > nf:
                    v = ns[k] * (zs[l] - z_low) / dz
                elif z_low < zmin_f:
                    v = ns[l] * (z_up - zs[l]) / dz
                else:
                    v = ns[k] * (zs[l] - z_low) / dz + ns[l] * (z_up - zs[l]) / dz
            out.append(v)
    norm = math.fsum(out) if False else sum(out)
    if norm == 0:
        raise ValueError("sum of n(z) is zero")
    norm *= dz
    return np.array([v / norm for v in out])


def theta_triplets(thetas):
    """All theta1<=theta2<=theta3 combinations in the reference's loop order
    (cuda_version/calculateApertureStatistics.cu:92-115)."""
    out = []
    n = len(thetas)
    for i in range(n):
        for j in range(i, n):
            for k in range(j, n):
                out.append((thetas[i], thetas[j], thetas[k]))
    return out


# ---------------------------------------------------------------------------
class Tables:
    """One cosmology's FP64 tables (set_cosmology) plus scalar physics."""

    def __init__(self, cosmo: dict, nz, pk=None, dk=0.0, kmin=0.0, kmax=0.0):
        L = lib()
        self.cosmo = dict(cosmo)
        c = Cosmo(**{k: float(cosmo[k]) for k in ("h", "sigma8", "omb", "omc", "ns", "w", "om", "ow", "zmax")})
        nz = np.ascontiguousarray(nz, dtype=np.float64)
        pkp = None
        if pk is not None:
            pk = np.ascontiguousarray(pk, dtype=np.float64)
            pkp = _dp(pk)
        self._h = L.orc_tables_create(C.byref(c), _dp(nz), pkp, dk, kmin, kmax)

    def __del__(self):
        try:
            lib().orc_tables_destroy(self._h)
        except Exception:
            pass

    def arrays(self):
        out = np.zeros(6 * NZ + 1)
        lib().orc_tables_get(self._h, _dp(out))
        names = ("f_K", "g", "D1", "r_sigma", "n_eff", "ncur")
        d = {n: out[i * NZ:(i + 1) * NZ].copy() for i, n in enumerate(names)}
        d["norm"] = out[6 * NZ]
        return d

    def set_noise(self, sigma, ngal, constant_ps=False):
        lib().orc_set_noise(self._h, sigma, ngal, int(constant_ps))

    def set_analytic(self, on=True):
        lib().orc_set_analytic(self._h, int(on))

    def __getattr__(self, name):
        L = lib()
        fn = getattr(L, "orc_" + name)
        return lambda *a: fn(self._h, *a)

    def bkappa_batch(self, ell):
        ell = np.ascontiguousarray(ell, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(ell))
        lib().orc_bkappa_batch(self._h, _dp(ell), len(ell), _dp(out))
        return out

    def map3(self, thetas, phiMin=0.0, phiMax=2 * math.pi, lMin=1.0, lMax=0.0, rel=1e-4):
        err = C.c_double(0)
        nev = C.c_long(0)
        th = np.array(thetas, dtype=np.float64)
        v = lib().orc_MapMapMap(self._h, _dp(th), phiMin, phiMax, lMin, lMax, rel, C.byref(err), C.byref(nev))
        return v, err.value, nev.value

    def gamma(self, comp, x1, x2, x3, rel=1e-3, abs_tol=0.0):
        re, im = C.c_double(0), C.c_double(0)
        nev = C.c_long(0)
        lib().orc_gamma(self._h, comp, x1, x2, x3, rel, abs_tol, C.byref(re), C.byref(im), C.byref(nev))
        return complex(re.value, im.value), nev.value

    def gamma_integrand_points(self, which, x1, x2, x3, pts):
        """Sum over the Ogata nodes of the Gamma^0 (which=0) or Gamma^1
        (which=1) integrand at points (z, phi, psi); complex array."""
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(2 * len(pts))
        lib().orc_gamma_integrand_points(self._h, which, x1, x2, x3, _dp(pts), len(pts), _dp(out))
        return out[0::2] + 1j * out[1::2]

    def cov_T(self, term, params: CovParams, th6, rel=0.0):
        th = np.array(th6, dtype=np.float64)
        nev = C.c_long(0)
        L = lib()
        if term == 1:
            return L.orc_T1(self._h, C.byref(params), _dp(th), rel, C.byref(nev)), nev.value
        if term == 2:
            return L.orc_T2(self._h, C.byref(params), _dp(th)), 0
        return L.orc_T4(self._h, C.byref(params), _dp(th), rel, C.byref(nev)), nev.value

    # ---- halo model (T5, T6, T7) ----
    def halo_tables(self):
        """sigma^2(m_i) and dsigma^2/dm(m_i) at z = 0, 128 masses each."""
        out = np.zeros(256)
        lib().orc_halo_tables(self._h, _dp(out))
        return out[:128].copy(), out[128:].copy()

    def halo_los(self, pts):
        """Line-of-sight one-halo trispectrum (l1..l4) and pentaspectrum
        (l1..l6) at rows (m, l1, ..., l6)."""
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 7)
        tri, pen = np.zeros(len(pts)), np.zeros(len(pts))
        lib().orc_halo_los(self._h, _dp(pts), len(pts), _dp(tri), _dp(pen))
        return tri, pen

    def halo_integrand(self, term, params: CovParams, th6, lmax, x):
        ndim = 6 if term == 5 else 7
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, ndim)
        th = np.array(th6, dtype=np.float64)
        out = np.zeros(len(x))
        lib().orc_halo_integrand(self._h, C.byref(params), term, _dp(th), lmax, _dp(x), len(x), _dp(out))
        return out

    def cov_T_halo(self, term, params: CovParams, th6, rel=0.0, max_eval=0):
        """T5/T6/T7 single term: (value, error estimate, evaluations)."""
        th = np.array(th6, dtype=np.float64)
        err, nev = C.c_double(0), C.c_long(0)
        v = lib().orc_T_halo(self._h, C.byref(params), term, _dp(th), rel, max_eval, C.byref(err), C.byref(nev))
        return v, err.value, nev.value

    def cov_total_halo(self, term, params: CovParams, th123, th456, rel=0.0, max_eval=0):
        a = np.array(th123, dtype=np.float64)
        b = np.array(th456, dtype=np.float64)
        return lib().orc_T_halo_total(self._h, C.byref(params), term, _dp(a), _dp(b), rel, max_eval)

    def cov_total(self, term, params: CovParams, th123, th456):
        a = np.array(th123, dtype=np.float64)
        b = np.array(th456, dtype=np.float64)
        fn = {1: lib().orc_T1_total, 2: lib().orc_T2_total, 4: lib().orc_T4_total}[term]
        return fn(self._h, C.byref(params), _dp(a), _dp(b))


def halo_total_terms(term, th123, th456):
    """(multiplicity, argument indices into (a0, a1, a2, b0, b1, b2)) of the
    reference's T5_total / T6_total / T7_total."""
    a = np.array(th123, dtype=np.float64)
    b = np.array(th456, dtype=np.float64)
    mult = (C.c_int * 16)()
    idx = (C.c_int * 96)()
    n = lib().orc_halo_total_terms(term, _dp(a), _dp(b), mult, idx)
    return [(mult[k], tuple(idx[6 * k:6 * k + 6])) for k in range(n)]


def sici(x):
    si, ci = C.c_double(0), C.c_double(0)
    lib().orc_sici(x, C.byref(si), C.byref(ci))
    return si.value, ci.value


def ogata_weights():
    out = np.zeros(4 * 33)
    lib().orc_ogata_weights(_dp(out))
    return out.reshape(4, 33)


def gq96():
    a, w = np.zeros(48), np.zeros(48)
    lib().orc_gq96(_dp(a), _dp(w))
    return a, w


def ggg_analytic(r1, r2, r3):
    re, im = C.c_double(0), C.c_double(0)
    lib().orc_ggg_analytic(r1, r2, r3, C.byref(re), C.byref(im))
    return complex(re.value, im.value)


def set_threads(n: int):
    lib().orc_set_threads(int(n))


# ---------------------------------------------------------------------------
# the reference's own host code (only where the reference tree was present at
# build time: oracle/_ref/libref_host.so)
# ---------------------------------------------------------------------------
_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB_PATH):
            return None
        L = C.CDLL(REF_LIB_PATH)
        d, p, i = C.c_double, C.c_void_p, C.c_int
        dp = C.POINTER(C.c_double)
        L.ref_set_cosmo.argtypes = [d] * 9
        L.ref_build_tables.argtypes = [dp, dp]
        for n, k in (("ref_lgr", 1), ("ref_calc_r_sigma", 1), ("ref_f_K_at_z", 1), ("ref_E", 1),
                     ("ref_linear_pk", 1), ("ref_P_k_nonlinear", 2), ("ref_limber_integrand", 2),
                     ("ref_GQ96_of_Pk", 1)):
            getattr(L, n).restype = d
            getattr(L, n).argtypes = [d] * k
        L.ref_sigmam.restype = d
        L.ref_sigmam.argtypes = [d, i]
        L.ref_g_interpolated.restype = d
        L.ref_g_interpolated.argtypes = [i, d]
        L.ref_f_K_interpolated.restype = d
        L.ref_f_K_interpolated.argtypes = [i, d]
        L.ref_compute_coefficients.argtypes = [i, d, dp]
        L.ref_gq96.argtypes = [dp, dp]
        L.ref_hcubature_v.restype = i
        L.ref_hcubature_v.argtypes = [C.c_uint, p, p, C.c_uint, dp, dp, C.c_size_t, d, d, i, dp, dp]
        if hasattr(L, "ref_halo_tables"):
            L.ref_halo_tables.argtypes = [dp]
            for n, k in (("ref_hmf", 2), ("ref_r_200", 2), ("ref_u_NFW", 3), ("ref_concentration", 2),
                         ("ref_get_sigma2", 2), ("ref_get_dSigma2dm", 2), ("ref_halo_bias", 2)):
                getattr(L, n).restype = d
                getattr(L, n).argtypes = [d] * k
            L.ref_SiCi.argtypes = [d, dp, dp]
        _ref = L
    return _ref
