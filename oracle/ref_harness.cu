// Thin C harness around the reference's own host code, used only to pin the
// oracle (test infrastructure; built by `make ref` into oracle/_ref/ from the
// read-only reference tree, never shipped).
//
// It exposes the reference's host functions from cuda_version/bispectrum.cu
// (lgr, sigmam, calc_r_sigma, f_K_at_z, linear_pk, P_k_nonlinear,
// GQ96_of_Pk, interpolation helpers) and its vendored hcubature_v. The table
// loop below mirrors set_cosmology (cuda_version/bispectrum.cu:148-212) minus
// the constant-memory uploads, which need a GPU.
//
// It also exposes the host side of the halo model (cuda_version/halomodel.cu):
// sigma2(m) and dSigma2dm(m) (:179-277, the 128-entry mass tables that
// setSigma2 / setdSigma2dm fill) and the __host__ __device__ functions hmf,
// SiCi, r_200, u_NFW, concentration, get_sigma2, get_dSigma2dm and halo_bias
// evaluated on the host after ref_halo_tables has filled the host arrays.
#include "bispectrum.cuh"
#include "cubature.h"
#include "halomodel.cuh"

#include <cstring>

double lgr(double z);
double sigmam(double r, int j);
double calc_r_sigma(double D1);
double f_K_at_z(double z);
double E(double z);
double GQ96_of_Pk(double a, double b, double ell);
double limber_integrand_power_spectrum(double ell, double z);
double P_k_nonlinear(double k, double z);
double linear_pk(double k);
double g_interpolated(int idx, double didx);
double f_K_interpolated(int idx, double didx);
void compute_coefficients(int idx, double didx, double* D1, double* r_sigma, double* n_eff, double* ncur);

// halomodel.cu's device code reads this survey-variance table, which
// apertureStatisticsCovariance.cu defines; that file is not compiled here.
__constant__ double dev_sigma2_from_windowfunction_array[n_redshift_bins];

extern "C" {

void ref_set_cosmo(double h, double sigma8, double omb, double omc, double ns, double w, double om, double ow,
                   double zmax) {
  cosmo.h = h;
  cosmo.sigma8 = sigma8;
  cosmo.omb = omb;
  cosmo.omc = omc;
  cosmo.ns = ns;
  cosmo.w = w;
  cosmo.om = om;
  cosmo.ow = ow;
  cosmo.zmax = zmax;
  Pk_given = false;
  norm_P = 1;
  norm_P = cosmo.sigma8 / sigmam(8., 0);
  z_max = cosmo.zmax;
  dz = z_max / n_redshift_bins;
}

// out: f_K, g, D1, r_sigma, n_eff, ncur (256 each), then norm_P
void ref_build_tables(const double* nz, double* out) {
  for (int i = 0; i < n_redshift_bins; i++) f_K_array[i] = f_K_at_z((i + 0.5) * dz);
  for (int i = 0; i < n_redshift_bins; i++) {
    g_array[i] = 0;
    for (int j = i; j < n_redshift_bins; j++) {
      if (j == i || j == n_redshift_bins - 1)
        g_array[i] += nz[j] * (f_K_array[j] - f_K_array[i]) / f_K_array[j] / 2;
      else
        g_array[i] += nz[j] * (f_K_array[j] - f_K_array[i]) / f_K_array[j];
    }
    g_array[i] = g_array[i] * dz;
  }
  g_array[0] = 1.;
  for (int i = 0; i < n_redshift_bins; i++) {
    double z_now = (i + 0.5) * dz;
    D1_array[i] = lgr(z_now) / lgr(0.);
    r_sigma_array[i] = calc_r_sigma(D1_array[i]);
    double d1 = -2. * pow(D1_array[i] * sigmam(r_sigma_array[i], 2), 2);
    n_eff_array[i] = -3. + 2. * pow(D1_array[i] * sigmam(r_sigma_array[i], 2), 2);
    ncur_array[i] = d1 * d1 + 4. * sigmam(r_sigma_array[i], 3) * pow(D1_array[i], 2);
  }
  const int n = n_redshift_bins;
  std::memcpy(out + 0 * n, f_K_array, sizeof(double) * n);
  std::memcpy(out + 1 * n, g_array, sizeof(double) * n);
  std::memcpy(out + 2 * n, D1_array, sizeof(double) * n);
  std::memcpy(out + 3 * n, r_sigma_array, sizeof(double) * n);
  std::memcpy(out + 4 * n, n_eff_array, sizeof(double) * n);
  std::memcpy(out + 5 * n, ncur_array, sizeof(double) * n);
  out[6 * n] = norm_P;
}

double ref_lgr(double z) { return lgr(z); }
double ref_sigmam(double r, int j) { return sigmam(r, j); }
double ref_calc_r_sigma(double D1) { return calc_r_sigma(D1); }
double ref_f_K_at_z(double z) { return f_K_at_z(z); }
double ref_E(double z) { return E(z); }
double ref_linear_pk(double k) { return linear_pk(k); }
double ref_P_k_nonlinear(double k, double z) { return P_k_nonlinear(k, z); }
double ref_limber_integrand(double ell, double z) { return limber_integrand_power_spectrum(ell, z); }
// the device Pell without shape noise: GQ96 over [0, z_max]
double ref_GQ96_of_Pk(double ell) { return GQ96_of_Pk(0, z_max, ell); }
double ref_g_interpolated(int idx, double didx) { return g_interpolated(idx, didx); }
double ref_f_K_interpolated(int idx, double didx) { return f_K_interpolated(idx, didx); }
void ref_compute_coefficients(int idx, double didx, double* out4) {
  compute_coefficients(idx, didx, &out4[0], &out4[1], &out4[2], &out4[3]);
}
void ref_gq96(double* a, double* w) {
  std::memcpy(a, A96, sizeof(double) * 48);
  std::memcpy(w, W96, sizeof(double) * 48);
}

int ref_hcubature_v(unsigned fdim, integrand_v f, void* fdata, unsigned dim, const double* xmin,
                    const double* xmax, size_t maxEval, double reqAbsError, double reqRelError, int norm,
                    double* val, double* err) {
  return hcubature_v(fdim, f, fdata, dim, xmin, xmax, maxEval, reqAbsError, reqRelError, (error_norm)norm, val,
                     err);
}

// setSigma2 / setdSigma2dm (halomodel.cu:197-214,262-276) without the
// constant-memory uploads: out[0..127] = sigma2(m_i), out[128..255] =
// dSigma2dm(m_i), m_i = 10^(logMmin + i (logMmax - logMmin) / n_mbins); the
// host arrays that get_sigma2 / get_dSigma2dm read are filled too
void ref_halo_tables(double* out) {
  const double deltaM = (logMmax - logMmin) / n_mbins;
  for (int i = 0; i < n_mbins; i++) {
    const double m = pow(10, logMmin + i * deltaM);
    sigma2_array[i] = sigma2(m);
    dSigma2dm_array[i] = dSigma2dm(m);
    out[i] = sigma2_array[i];
    out[n_mbins + i] = dSigma2dm_array[i];
  }
}
double ref_hmf(double m, double z) { return hmf(m, z); }
void ref_SiCi(double x, double* si, double* ci) { SiCi(x, *si, *ci); }
double ref_r_200(double m, double z) { return r_200(m, z); }
double ref_u_NFW(double k, double m, double z) { return u_NFW(k, m, z); }
double ref_concentration(double m, double z) { return concentration(m, z); }
double ref_get_sigma2(double m, double z) { return get_sigma2(m, z); }
double ref_get_dSigma2dm(double m, double z) { return get_dSigma2dm(m, z); }
double ref_halo_bias(double m, double z) { return halo_bias(m, z); }
}
