// The reference's C++ API (cuda_version/*.cuh of sheydenreich/threepoint) as
// inline functions over the C ABI of libthreepoint_gb300.so, so that C++ code
// written against the reference compiles and links unchanged (link with
// -lthreepoint_gb300). Header-only, C++17.
//
// Same names, argument meaning and globals as the reference:
//   cosmology (cosmology.cuh:13-29), read_n_of_z, read_thetas,
//   convert_angle_to_rad, convert_rad_to_angle (helpers.cuh:21-40),
//   copyConstants, set_cosmology (bispectrum.cuh:81,92),
//   MapMapMap (apertureStatistics.cuh:106),
//   gamma0..gamma3, compute_weights_bessel (gamma.cuh:56-97,291),
//   the covariance globals type, thetaMax, thetaMax_smaller, area, lMin,
//   sigma, n, constant_powerspectrum and initCovariance, T1_total, T2_total,
//   T4_total, T5_total, T6_total, T7_total, T7_2h_total, initHalomodel
//   (apertureStatisticsCovariance.cuh:22-54,116-136; bispectrum.cuh:19,29;
//   halomodel.cuh).
// Differences: errors throw std::runtime_error (or std::invalid_argument)
// where the reference prints and calls exit(); all evaluations are FP64 (the
// reference's arithmetic); gamma*'s z_max must be the cosmology's zmax (the
// value every reference driver passes); covariance terms need lMin == 0 (the
// value calculateApertureStatisticsCovariance sets). The GPU is
// threepoint_device (default 0), one cosmology at a time as in the reference.
#pragma once
#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "threepoint_gb300.h"

// ---- globals of the reference ---------------------------------------------
inline int threepoint_device = 0;  // CUDA device used by this API (not in the reference)
inline int type = 1;               // 0 circle, 1 square, 2 infinite, 3 rectangular
inline double thetaMax = 0;        // [rad] survey radius (circle) or side (square, rectangle)
inline double thetaMax_smaller = 0;  // [rad] smaller side of a rectangle
inline double area = 0;            // [rad^2]
inline double lMin = 0;            // lower ell bound of the covariance integrals
inline double sigma = 0, n = 1;    // shape noise and galaxy number density [rad^-2]
inline bool constant_powerspectrum = false;  // shape-noise-only P(ell)
inline double z_max = 0;           // zmax of the current cosmology

namespace threepoint_gb300_detail {
inline tp_ctx*& ctx() {
  static tp_ctx* c = nullptr;
  return c;
}
inline tp_cosmology& cosmo() {
  static tp_cosmology c{};
  return c;
}
inline bool& have_cosmo() {
  static bool h = false;
  return h;
}
inline void check(int st, const char* what) {
  if (st == TP_OK) return;
  std::string msg = std::string(what) + ": " + tp_status_string(st);
  if (ctx() && tp_last_error(ctx())[0]) msg += " (" + std::string(tp_last_error(ctx())) + ")";
  throw std::runtime_error(msg);
}
inline tp_ctx* need_ctx() {
  if (!ctx()) check(tp_ctx_create(threepoint_device, &ctx()), "copyConstants");
  return ctx();
}
inline void need_cosmo(const char* what) {
  if (!have_cosmo()) throw std::runtime_error(std::string(what) + ": set_cosmology has not been called");
}
}  // namespace threepoint_gb300_detail

// ---- cosmology and inputs ----------------------------------------------------
class cosmology {
 public:
  double h = 0, sigma8 = 0, omb = 0, omc = 0, ns = 0, w = 0, om = 0, ow = 0, zmax = 0;
  cosmology() {}
  explicit cosmology(const std::string& fn_parameters) {
    tp_cosmology c;
    threepoint_gb300_detail::check(tp_cosmology_from_file(fn_parameters.c_str(), &c), "cosmology");
    h = c.h, sigma8 = c.sigma8, omb = c.omb, omc = c.omc, ns = c.ns, w = c.w, om = c.om, ow = c.ow, zmax = c.zmax;
  }
};

inline void read_n_of_z(const std::string& fn, const int& n_bins, const double& zMax, std::vector<double>& nz) {
  std::vector<double> v(n_bins);
  threepoint_gb300_detail::check(tp_read_n_of_z(fn.c_str(), n_bins, zMax, v.data()), "read_n_of_z");
  nz = v;
}

inline void read_thetas(const std::string& fn, std::vector<double>& thetas) {
  std::vector<double> v(1 << 16);
  int cnt = 0;
  threepoint_gb300_detail::check(tp_read_thetas(fn.c_str(), v.data(), (int)v.size(), &cnt), "read_thetas");
  v.resize(cnt < (int)v.size() ? cnt : v.size());
  thetas.insert(thetas.end(), v.begin(), v.end());
}

inline double convert_angle_to_rad(const double& value, const std::string& unit = "arcmin") {
  double r;
  if (tp_convert_angle_to_rad(value, unit.c_str(), &r) != TP_OK)
    throw std::invalid_argument("Unit not correctly specified. Needs to be arcmin, deg, or rad.");
  return r;
}

// helpers.cu:155-174: the factors 3437.74677 (arcmin) and 57.3 (deg)
inline double convert_rad_to_angle(const double& value, const std::string& unit = "arcmin") {
  if (unit == "arcmin") return 3437.74677 * value;
  if (unit == "deg") return 57.3 * value;
  throw std::invalid_argument("Unit not correctly specified. Needs to be arcmin or deg.");
}

// ---- set-up --------------------------------------------------------------------
inline void copyConstants() { threepoint_gb300_detail::need_ctx(); }

inline void set_cosmology(cosmology c, std::vector<double>* nz = nullptr, std::vector<double>* P_k = nullptr,
                          double dk = 0, double kmin = 0, double kmax = 1e4) {
  using namespace threepoint_gb300_detail;
  if (!nz) throw std::invalid_argument("set_cosmology: No n(z) given");  // the reference exits here
  if (nz->size() != 256) throw std::invalid_argument("set_cosmology: n(z) needs 256 bins");
  if (P_k && P_k->size() != 256) throw std::invalid_argument("set_cosmology: P(k) needs 256 bins");
  tp_cosmology t{c.h, c.sigma8, c.omb, c.omc, c.ns, c.w, c.om, c.ow, c.zmax};
  check(tp_set_cosmologies(need_ctx(), &t, 1, nz->data(), 0, P_k ? P_k->data() : nullptr, dk, kmin, kmax),
        "set_cosmology");
  cosmo() = t;
  have_cosmo() = true;
  z_max = c.zmax;
}

// ---- <Map^3> -------------------------------------------------------------------
inline double MapMapMap(const std::vector<double>& thetas, const double& phiMin = 0, const double& phiMax = 2 * M_PI,
                        const double& lMin_ = 1) {
  using namespace threepoint_gb300_detail;
  need_cosmo("MapMapMap");
  if (thetas.size() != 3) throw std::invalid_argument("MapMapMap: needs three aperture radii");
  double out = 0;
  int st = tp_map3_batch(ctx(), nullptr, 1, thetas.data(), 1, phiMin, phiMax, lMin_, 0.0, 1e-4, TP_FP64, &out,
                         nullptr, nullptr, nullptr);
  if (st != TP_ERR_CAPACITY) check(st, "MapMapMap");  // a capped integral still returns its value
  return out;
}

// ---- shear 3PCF ------------------------------------------------------------------
inline void compute_weights_bessel() {}  // the Ogata nodes are built by the library

namespace threepoint_gb300_detail {
inline std::complex<double> gamma_k(int k, double x1, double x2, double x3, double zmax) {
  need_cosmo("gamma");
  if (std::fabs(zmax - cosmo().zmax) > 1e-12 * std::fabs(cosmo().zmax))
    throw std::invalid_argument("gamma: z_max must be the cosmology's zmax");
  const double x[3] = {x1, x2, x3};
  double out[8] = {0};
  int st = tp_gamma_batch(ctx(), 0, x, 1, 1 << k, 1e-3, TP_FP64, out, nullptr);
  if (st != TP_ERR_CAPACITY) check(st, "gamma");
  return {out[2 * k], out[2 * k + 1]};
}

inline double cov_total(int term, const std::vector<double>& a, const std::vector<double>& b) {
  need_cosmo("T_total");
  if (a.size() != 3 || b.size() != 3) throw std::invalid_argument("T_total: Wrong number of aperture radii");
  if (lMin != 0) throw std::invalid_argument("T_total: only lMin = 0 is supported");
  check(tp_set_shape_noise(ctx(), sigma, n, constant_powerspectrum), "initCovariance");
  if (type == 3) check(tp_set_rectangle_side(ctx(), thetaMax_smaller), "initCovariance");
  double out = 0;
  int capped = 0;
  int st = tp_cov_total_batch(ctx(), 0, term, type, thetaMax, area, a.data(), b.data(), 1, TP_FP64, &out, &capped);
  if (st != TP_ERR_CAPACITY) check(st, "T_total");
  return out;
}
}  // namespace threepoint_gb300_detail

inline std::complex<double> gamma0(double x1, double x2, double x3, double zmax) {
  return threepoint_gb300_detail::gamma_k(0, x1, x2, x3, zmax);
}
inline std::complex<double> gamma1(double x1, double x2, double x3, double zmax) {
  return threepoint_gb300_detail::gamma_k(1, x1, x2, x3, zmax);
}
inline std::complex<double> gamma2(double x1, double x2, double x3, double zmax) {
  return threepoint_gb300_detail::gamma_k(2, x1, x2, x3, zmax);
}
inline std::complex<double> gamma3(double x1, double x2, double x3, double zmax) {
  return threepoint_gb300_detail::gamma_k(3, x1, x2, x3, zmax);
}

// ---- <Map^3> covariance ------------------------------------------------------------
// initCovariance copies the globals; T*_total also read them at each call.
inline void initCovariance() {
  using namespace threepoint_gb300_detail;
  check(tp_set_shape_noise(need_ctx(), sigma, n, constant_powerspectrum), "initCovariance");
  if (type == 3) check(tp_set_rectangle_side(ctx(), thetaMax_smaller), "initCovariance");
}
inline double T1_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(1, thetas_123, thetas_456);
}
inline double T2_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(2, thetas_123, thetas_456);
}
inline double T4_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(4, thetas_123, thetas_456);
}
// halo-model terms (apertureStatisticsCovariance.cu:685-1044); the halo model
// (initHalomodel, halomodel.cu:18-29) is built on first use
inline void initHalomodel() {}
inline double T5_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(5, thetas_123, thetas_456);
}
inline double T6_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(6, thetas_123, thetas_456);
}
inline double T7_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  return threepoint_gb300_detail::cov_total(7, thetas_123, thetas_456);
}
// T7_2h_total (apertureStatisticsCovariance.cu:1046-1063, 1315-1356): 0 for the
// infinite survey; for the square the reference's integrand multiplies by a
// survey-variance table it never fills (dev_sigma2_from_windowfunction_array),
// so its value is 0 as well; the other geometries throw, as the reference does.
inline double T7_2h_total(const std::vector<double>& thetas_123, const std::vector<double>& thetas_456) {
  if (thetas_123.size() != 3 || thetas_456.size() != 3)
    throw std::invalid_argument("T7_2h_total: Wrong number of aperture radii");
  if (type == 2 || type == 1) return 0.0;
  throw std::logic_error("T7_SSC: Wrong survey geometry, only coded for square survey");
}
