// CPU FP64 oracle for the threepoint model-evaluation path.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker: it is loaded by the
// tests, by the smoke check and by the CPU-baseline leg of the benchmark, and
// never by the product library (threepoint_gb300/), which has no CPU fallback.
//
// It restates, in plain C++17 double precision, the semantics of the
// reference's cuda_version tree (file:line citations at each function), with
// one deliberate fix: the mid-bin interpolation clamps the lower neighbour to
// bin 0 where the reference reads index -1 (cuda_version/bispectrum.cu:356-359,
// 389-392, 421-424).
#pragma once
#include <cstddef>

extern "C" {

// cosmology block (cuda_version/cosmology.cuh:13-29)
typedef struct {
  double h, sigma8, omb, omc, ns, w, om, ow, zmax;
} orc_cosmo;

// integrand signature of the reference's cubature library (cubature.h)
typedef int (*orc_integrand_v)(unsigned ndim, size_t npts, const double* x,
                               void* fdata, unsigned fdim, double* fval);

enum { ORC_ERROR_INDIVIDUAL = 0, ORC_ERROR_PAIRED, ORC_ERROR_L2, ORC_ERROR_L1, ORC_ERROR_LINF };

// ---- tables (set_cosmology, cuda_version/bispectrum.cu:100-219) ----------
typedef struct orc_tables orc_tables;
// nz: 256 values on bins i*dz (output of read_n_of_z). pk: optional 256-bin
// log-spaced linear P(k) table (nullptr -> Eisenstein & Hu).
orc_tables* orc_tables_create(const orc_cosmo* c, const double* nz, const double* pk,
                              double dk, double kmin, double kmax);
void orc_tables_destroy(orc_tables* t);
// out: 6*256 doubles (f_K, g, D1, r_sigma, n_eff, ncur) followed by norm.
void orc_tables_get(const orc_tables* t, double* out);
void orc_set_noise(orc_tables* t, double sigma, double ngal, int constant_ps);
// analytic Gaussian-bispectrum test mode for the shear 3PCF
// (classed_version/bispectrum.cpp:477-499)
void orc_set_analytic(orc_tables* t, int on);

// ---- scalar physics --------------------------------------------------------
double orc_E(const orc_tables* t, double z);
double orc_linear_pk(const orc_tables* t, double k);
double orc_sigmam(const orc_tables* t, double r, int j);
double orc_lgr(const orc_tables* t, double z);
double orc_calc_r_sigma(const orc_tables* t, double D1);
double orc_f_K_at_z(const orc_tables* t, double z);
double orc_P_k_nonlinear(const orc_tables* t, double k, double z);
double orc_bispec_at_z(const orc_tables* t, double k1, double k2, double k3, double z);
double orc_integrand_bkappa(const orc_tables* t, double z, double l1, double l2, double l3);
double orc_bkappa(const orc_tables* t, double l1, double l2, double l3);
void orc_bkappa_batch(const orc_tables* t, const double* ell, long n, double* out);
double orc_Pell(const orc_tables* t, double ell);
double orc_limber_integrand(const orc_tables* t, double ell, double z);
double orc_uHat(double eta);
// 96-point Gauss-Legendre nodes/weights on (0,1) half (48 each), ascending
void orc_gq96(double* abscissa48, double* weight48);

// ---- cubature --------------------------------------------------------------
// Gladwell-parallel h-adaptive cubature with the Genz-Malik 7/5 rule (dim>=2)
// or Gauss-Kronrod 15 (dim=1); restatement of hcubature_v
// (cuda_version/hcubature.cpp:456-617, 620-780, 904-1067; converged.h).
int orc_hcubature_v(unsigned fdim, orc_integrand_v f, void* fdata, unsigned dim,
                    const double* xmin, const double* xmax, size_t maxEval,
                    double reqAbsError, double reqRelError, int norm, double* val,
                    double* err);
// number of integrand points evaluated by the last orc_hcubature_v on this thread
long orc_last_neval(void);

// ---- <Map^3> (cuda_version/apertureStatistics.cu:138-153,201-230) ----------
typedef struct orc_map3_ctx orc_map3_ctx;
orc_map3_ctx* orc_map3_ctx_create(const orc_tables* t, double th1, double th2, double th3);
void orc_map3_ctx_destroy(orc_map3_ctx* c);
int orc_integrand_map3_v(unsigned ndim, size_t npts, const double* x, void* fdata,
                         unsigned fdim, double* fval);
// lMax<=0 selects the reference bound 10/theta_min.
double orc_MapMapMap(const orc_tables* t, const double* thetas, double phiMin, double phiMax,
                     double lMin, double lMax, double relTol, double* err, long* neval);

// ---- shear 3PCF (cuda_version/gamma.cu) -----------------------------------
// ogata: 4*33 doubles: psi_J6, product_J6, psi_J2, product_J2 (index k=0..32)
void orc_ogata_weights(double* out);
// comp 0..3; returns complex via re/im; centroid conversion applied as in the
// reference build (CONVERT_TO_CENTROID defined, gamma.cuh:25).
void orc_gamma(const orc_tables* t, int comp, double x1, double x2, double x3,
               double relTol, double absTol, double* re, double* im, long* neval);
// closed-form Gamma^0 of the analytic test bispectrum
// (classed_version/gamma.cpp:83-93,567-582)
void orc_ggg_analytic(double r1, double r2, double r3, double* re, double* im);
// Ogata step h and node count (default 0.1 and 33, the CUDA settings)
void orc_set_ogata(double h, int nk);

// ---- <Map^3> covariance (cuda_version/apertureStatisticsCovariance.cu) ----
typedef struct {
  int type;          // 0 circle, 1 square, 2 infinite, 3 rectangular
  double thetaMax;   // rad
  double area;       // rad^2
  double lMin;       // integration lower bound used by T1 (infinite) and T2
  double thetaMaxSmaller;  // rad, second side of the rectangle (type 3)
} orc_cov_params;
double orc_T1(const orc_tables* t, const orc_cov_params* p, const double* th6, double relTol, long* neval);
double orc_T2(const orc_tables* t, const orc_cov_params* p, const double* th6);
double orc_T4(const orc_tables* t, const orc_cov_params* p, const double* th6, double relTol, long* neval);
double orc_T1_total(const orc_tables* t, const orc_cov_params* p, const double* th123, const double* th456);
double orc_T2_total(const orc_tables* t, const orc_cov_params* p, const double* th123, const double* th456);
double orc_T4_total(const orc_tables* t, const orc_cov_params* p, const double* th123, const double* th456);
double orc_G_square(double thetaMax, double lx, double ly);

void orc_set_threads(int n);
}
