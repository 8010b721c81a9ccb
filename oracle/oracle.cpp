// CPU FP64 oracle for the threepoint model-evaluation path.
//
// TEST INFRASTRUCTURE ONLY: the checker used by tests/, __graft_entry__.smoke()
// and the cpu_baseline leg of bench.py. The product never links or loads it.
//
// Semantics follow the reference's cuda_version tree; every function cites the
// reference file:line it restates. The one deliberate departure: the mid-bin
// table interpolation clamps the lower neighbour at bin 0, where the reference
// reads index -1 (cuda_version/bispectrum.cu:356-359,389-392,421-424).
#include "oracle.hpp"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int NZ = 256;   // n_redshift_bins, cuda_version/bispectrum.cuh:35
constexpr int NK = 256;   // n_kbins, cuda_version/bispectrum.cuh:37
constexpr double EPS = 1.0e-4;  // eps, cuda_version/bispectrum.cu:26
constexpr double H0_OVER_C = 100. / 299792.;  // bispectrum.cuh:60
constexpr double C_OVER_H0 = 2997.92;         // bispectrum.cuh:62
constexpr double PI = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// 96-point Gauss-Legendre rule on [-1,1], computed by Newton iteration on the
// Legendre polynomial (the reference hard-codes the same rule to 15 digits,
// cuda_version/bispectrum.cu:47-73).
struct GQ96 {
  double a[48], w[48];
  GQ96() {
    const int n = 96;
    for (int i = 0; i < 48; ++i) {
      // root number (48 - i) counted from x=0 upwards so that a[] ascends
      long double x = cosl(3.14159265358979323846264338327950288L * (47 - i + 1 - 0.25L) / (n + 0.5L));
      long double dp = 0;
      for (int it = 0; it < 100; ++it) {
        long double p0 = 1, p1 = x;
        for (int k = 2; k <= n; ++k) {
          long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (x * p1 - p0) / (x * x - 1);
        long double dx = p1 / dp;
        x -= dx;
        if (fabsl(dx) < 1e-19L) break;
      }
      {
        long double p0 = 1, p1 = x;
        for (int k = 2; k <= n; ++k) {
          long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
          p0 = p1;
          p1 = p2;
        }
        dp = n * (x * p1 - p0) / (x * x - 1);
      }
      a[i] = (double)x;
      w[i] = (double)(2.0L / ((1 - x * x) * dp * dp));
    }
  }
};
const GQ96& gq96() {
  static GQ96 g;
  return g;
}

}  // namespace

// ---------------------------------------------------------------------------
struct orc_tables {
  orc_cosmo c{};
  double norm = 1;  // norm_P
  double dz = 0, z_max = 0;
  double f_K[NZ], g[NZ], D1[NZ], r_sigma[NZ], n_eff[NZ], ncur[NZ];
  bool pk_given = false;
  double pk[NK];
  double dk = 0, kmin = 0, kmax = 0;
  double sigma = 0, ngal = 1;
  bool constant_ps = false;
  bool analytic = false;
  // halo model mass tables (sigma^2(m), dsigma^2/dm at z = 0), built on first use
  bool halo = false;
  double sig2[128], dsig2[128];
};

namespace {

// E(z), flat wCDM, cuda_version/bispectrum.cu:921-928
double E(const orc_tables* t, double z) {
  const orc_cosmo& c = t->c;
  return sqrt(c.om * pow(1 + z, 3) + c.ow * pow(1 + z, 3 * (1.0 + c.w)));
}
double E_inv(const orc_tables* t, double z) { return 1. / E(t, z); }

// bispectrum.cu:905-919
double GQ96_of_Einv(const orc_tables* t, double a, double b) {
  const GQ96& G = gq96();
  double cx = (a + b) / 2, dx = (b - a) / 2, q = 0;
  for (int i = 0; i < 48; i++) q += G.w[i] * (E_inv(t, cx - dx * G.a[i]) + E_inv(t, cx + dx * G.a[i]));
  return q * dx;
}

// bispectrum.cu:721-724
double f_K_at_z(const orc_tables* t, double z) { return C_OVER_H0 * GQ96_of_Einv(t, 0, z); }

// Eisenstein & Hu no-wiggle linear P(k) or table lookup, bispectrum.cu:602-693
double linear_pk(const orc_tables* t, double k) {
  if (t->pk_given) {
    if (k >= t->kmax) return t->pk[NK - 1];
    if (k <= t->kmin) return t->pk[0];
    double didx = log(k / t->kmin) / t->dk;
    int idx = (int)didx;
    didx = didx - idx;
    if (idx == NK - 1) return t->pk[NK - 1];
    return t->pk[idx] * (1 - didx) + t->pk[idx + 1] * didx;
  }
  const orc_cosmo& c = t->c;
  k *= c.h;
  double fc = c.omc / c.om, fb = c.omb / c.om;
  double theta = 2.728 / 2.7;
  double pc = 0.25 * (5.0 - sqrt(1.0 + 24.0 * fc));
  double omh2 = c.om * c.h * c.h, ombh2 = c.omb * c.h * c.h;
  double zeq = 2.5e+4 * omh2 / pow(theta, 4);
  double b1 = 0.313 * pow(omh2, -0.419) * (1.0 + 0.607 * pow(omh2, 0.674));
  double b2 = 0.238 * pow(omh2, 0.223);
  double zd = 1291.0 * pow(omh2, 0.251) / (1.0 + 0.659 * pow(omh2, 0.828)) * (1.0 + b1 * pow(ombh2, b2));
  double yd = (1.0 + zeq) / (1.0 + zd);
  double sh = 44.5 * log(9.83 / (omh2)) / sqrt(1.0 + 10.0 * pow(ombh2, 0.75));
  double alnu = fc * (5.0 - 2.0 * pc) / 5.0 * (1.0 - 0.553 * fb + 0.126 * fb * fb * fb) * pow(1.0 + yd, -pc) *
                (1.0 + 0.5 * pc * (1.0 + 1.0 / (7.0 * (3.0 - 4.0 * pc))) / (1.0 + yd));
  double geff = omh2 * (sqrt(alnu) + (1.0 - sqrt(alnu)) / (1.0 + pow(0.43 * k * sh, 4)));
  double qeff = k / geff * theta * theta;
  double L = log(2.718281828 + 1.84 * sqrt(alnu) * qeff / (1.0 - 0.949 * fb));
  double C = 14.4 + 325.0 / (1.0 + 60.5 * pow(qeff, 1.11));
  double delk = pow(t->norm, 2) * pow(k * 2997.9 / c.h, 3. + c.ns) * pow(L / (L + C * qeff * qeff), 2);
  double pk = 2.0 * PI * PI / (k * k * k) * delk;
  return c.h * c.h * c.h * pk;
}

// window functions, bispectrum.cu:854-868
double window(double x, int i) {
  if (i == 0) return 3.0 / pow(x, 3) * (sin(x) - x * cos(x));
  if (i == 1) return exp(-0.5 * x * x);
  if (i == 2) return x * exp(-0.5 * x * x);
  if (i == 3) return x * x * (1 - x * x) * exp(-x * x);
  if (i == 4) return (3 * (x * x - 3) * sin(x) + 9 * x * cos(x)) / x / x / x / x;
  return -1;
}

// sigma(R) by nested doubling trapezoid in ln k, bispectrum.cu:796-852
double sigmam(const orc_tables* t, double r, int j) {
  if (t->c.sigma8 < 1e-8) return 0;
  double k1 = 2. * PI / r, k2 = 2. * PI / r;
  double xx = 0, xxp, xxpp = -1.0;
  for (;;) {
    k1 = k1 / 10.0;
    k2 = k2 * 2.0;
    double a = log(k1), b = log(k2);
    xxp = -1.0;
    int n = 2;
    for (;;) {
      n = n * 2;
      double hh = (b - a) / (double)n;
      xx = 0.;
      for (int i = 1; i < n; i++) {
        double k = exp(a + hh * i);
        if (j < 3)
          xx += k * k * k * linear_pk(t, k) * pow(window(k * r, j), 2);
        else
          xx += k * k * k * linear_pk(t, k) * window(k * r, j);
      }
      if (j < 3)
        xx += 0.5 * (k1 * k1 * k1 * linear_pk(t, k1) * pow(window(k1 * r, j), 2) +
                     k2 * k2 * k2 * linear_pk(t, k2) * pow(window(k2 * r, j), 2));
      else
        xx += 0.5 * (k1 * k1 * k1 * linear_pk(t, k1) * window(k1 * r, j) +
                     k2 * k2 * k2 * linear_pk(t, k2) * window(k2 * r, j));
      xx *= hh;
      if (fabs((xx - xxp) / xx) < EPS) break;
      xxp = xx;
    }
    if (fabs((xx - xxpp) / xx) < EPS) break;
    xxpp = xx;
  }
  if (j < 3) return sqrt(xx / (2.0 * PI * PI));
  return xx / (2.0 * PI * PI);
}

// growth ODE right-hand side, bispectrum.cu:778-794
double lgr_func(const orc_tables* t, int j, double la, const double y[2]) {
  if (j == 0) return y[1];
  const orc_cosmo& c = t->c;
  double a = exp(la);
  double g = -0.5 * (5. * c.om + (5. - 3 * c.w) * c.ow * pow(a, -3. * c.w)) * y[1] -
             1.5 * (1. - c.w) * c.ow * pow(a, -3. * c.w) * y[0];
  return g / (c.om + c.ow * pow(a, -3. * c.w));
}

// linear growth by RK4 with step doubling, bispectrum.cu:726-776
double lgr(const orc_tables* t, double z) {
  double a = 1. / (1. + z), a0 = 1. / 1100.;
  double yp = -1.;
  int n = 10;
  double y[2], y2[2], y3[2], y4[2], k1[2], k2[2], k3[2], k4[2];
  for (;;) {
    n *= 2;
    double h = (log(a) - log(a0)) / n;
    double x = log(a0);
    y[0] = 1., y[1] = 0.;
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < 2; j++) k1[j] = h * lgr_func(t, j, x, y);
      for (int j = 0; j < 2; j++) y2[j] = y[j] + 0.5 * k1[j];
      for (int j = 0; j < 2; j++) k2[j] = h * lgr_func(t, j, x + 0.5 * h, y2);
      for (int j = 0; j < 2; j++) y3[j] = y[j] + 0.5 * k2[j];
      for (int j = 0; j < 2; j++) k3[j] = h * lgr_func(t, j, x + 0.5 * h, y3);
      for (int j = 0; j < 2; j++) y4[j] = y[j] + k3[j];
      for (int j = 0; j < 2; j++) k4[j] = h * lgr_func(t, j, x + h, y4);
      for (int j = 0; j < 2; j++) y[j] += (k1[j] + k4[j]) / 6. + (k2[j] + k3[j]) / 3.;
      x += h;
    }
    if (fabs(y[0] / yp - 1.) < 0.1 * EPS) break;
    yp = y[0];
  }
  return a * y[0];
}

// r_sigma = 1/k_sigma by bisection on D1*sigma(1/k)=1, bispectrum.cu:870-903
double calc_r_sigma(const orc_tables* t, double D1) {
  if (t->c.sigma8 < 1e-8) return 0;
  double k, k1, k2;
  k1 = k2 = 1.;
  for (;;) {
    if (D1 * sigmam(t, 1. / k1, 1) < 1.) break;
    k1 *= 0.5;
  }
  for (;;) {
    if (D1 * sigmam(t, 1. / k2, 1) > 1.) break;
    k2 *= 2.;
  }
  for (;;) {
    k = 0.5 * (k1 + k2);
    double s = D1 * sigmam(t, 1. / k, 1);
    if (s < 1.)
      k1 = k;
    else if (s > 1.)
      k2 = k;
    if (s == 1. || fabs(k2 / k1 - 1.) < EPS * 0.1) break;
  }
  return 1. / k;
}

// Mid-bin two-point interpolation of a z table (bispectrum.cu:335-437), with
// the lower neighbour clamped to bin 0.
inline void interp_weights(int idx, double didx, int& iidx, double& w, double& iw) {
  iidx = idx;
  w = 1 - fabs(didx - 0.5);
  iw = 1 - w;
  if (didx > 0.5) {
    if (idx == NZ - 1) {
      iidx = idx;
      iw = 0.0;
    } else {
      iidx = idx + 1;
    }
  } else if (didx < 0.5) {
    iidx = idx - 1 < 0 ? 0 : idx - 1;
  }
}
inline double interp(const double* arr, int idx, double didx) {
  int ii;
  double w, iw;
  interp_weights(idx, didx, ii, w, iw);
  return arr[idx] * w + arr[ii] * iw;
}
inline void clamp_idx(int& idx, double& didx) {
  if (idx > NZ - 1) {  // z beyond z_max never occurs on the reference's grids
    idx = NZ - 1;
    didx = 1.0;
  }
}

// Omega_m(z), Omega_Lambda(z), bispectrum.cu:439-457
double om_m_of_z(const orc_tables* t, double z) {
  double aa = 1. / (1 + z);
  const orc_cosmo& c = t->c;
  return c.om / (c.om + aa * (aa * aa * c.ow + (1. - c.om - c.ow)));
}
double om_v_of_z(const orc_tables* t, double z) {
  double aa = 1. / (1 + z);
  const orc_cosmo& c = t->c;
  return c.ow * aa * aa * aa / (c.om + aa * (aa * aa * c.ow + (1. - c.om - c.ow)));
}

// revised Halofit P(k,z), bispectrum.cu:531-600
double P_k_nonlinear(const orc_tables* t, double k, double z) {
  double didx = z / t->z_max * (NZ - 1);
  int idx = (int)didx;
  didx = didx - idx;
  clamp_idx(idx, didx);
  double D1 = interp(t->D1, idx, didx), r_sigma = interp(t->r_sigma, idx, didx);
  double n_eff = interp(t->n_eff, idx, didx), ncur = interp(t->ncur, idx, didx);
  double nsqr = n_eff * n_eff;
  double w = t->c.w;
  double om_m = om_m_of_z(t, z), om_v = om_v_of_z(t, z);
  double f1a = pow(om_m, (-0.0732)), f2a = pow(om_m, (-0.1423)), f3a = pow(om_m, (0.0725));
  double f1b = pow(om_m, (-0.0307)), f2b = pow(om_m, (-0.0585)), f3b = pow(om_m, (0.0743));
  double frac = om_v / (1. - om_m);
  double f1 = frac * f1b + (1 - frac) * f1a;
  double f2 = frac * f2b + (1 - frac) * f2a;
  double f3 = frac * f3b + (1 - frac) * f3a;
  double a = 1.5222 + 2.8553 * n_eff + 2.3706 * nsqr + 0.9903 * n_eff * nsqr + 0.2250 * nsqr * nsqr -
             0.6038 * ncur + 0.1749 * om_v * (1.0 + w);
  a = pow(10.0, a);
  double b = pow(10.0, -0.5642 + 0.5864 * n_eff + 0.5716 * nsqr - 1.5474 * ncur + 0.2279 * om_v * (1.0 + w));
  double c = pow(10.0, 0.3698 + 2.0404 * n_eff + 0.8161 * nsqr + 0.5869 * ncur);
  double gam = 0.1971 - 0.0843 * n_eff + 0.8460 * ncur;
  double alpha = fabs(6.0835 + 1.3373 * n_eff - 0.1959 * nsqr - 5.5274 * ncur);
  double beta = 2.0379 - 0.7354 * n_eff + 0.3157 * nsqr + 1.2490 * n_eff * nsqr + 0.3980 * nsqr * nsqr -
                0.1682 * ncur;
  double xnu = pow(10.0, 5.2105 + 3.6902 * n_eff);
  double plin = linear_pk(t, k) * D1 * D1 * k * k * k / (2 * PI * PI);
  double y = k * r_sigma, ysqr = y * y;
  double ph = a * pow(y, f1 * 3) / (1 + b * pow(y, f2) + pow(f3 * c * y, 3 - gam));
  ph = ph / (1 + xnu / ysqr);
  double pq = plin * pow(1 + plin, beta) / (1 + plin * alpha) * exp(-y / 4.0 - ysqr / 8.0);
  return 2 * PI * PI * (pq + ph) / (k * k * k);
}

// tree-level F2 and BiHalofit F2, bispectrum.cu:700-719
double F2_tree(double k1, double k2, double k3) {
  double c12 = 0.5 * (k3 * k3 - k1 * k1 - k2 * k2) / (k1 * k2);
  return (5. / 7.) + 0.5 * c12 * (k1 / k2 + k2 / k1) + (2. / 7.) * c12 * c12;
}
double F2(const orc_tables* t, double k1, double k2, double k3, double z, double D1, double r_sigma) {
  const orc_cosmo& c = t->c;
  double q3 = k3 * r_sigma;
  double logsigma8z = log10(D1 * c.sigma8);
  double a = 1. / (1. + z);
  double omz = c.om / (c.om + c.ow * pow(a, -3. * c.w));
  double dn = pow(10., -0.483 + 0.892 * logsigma8z - 0.086 * omz);
  return F2_tree(k1, k2, k3) + dn * q3;
}

// BiHalofit bispectrum (Takahashi+2020 B4-B9), bispectrum.cu:221-291,695-698
double bispec(const orc_tables* t, double k1, double k2, double k3, double z, int idx, double didx) {
  const orc_cosmo& c = t->c;
  double D1 = interp(t->D1, idx, didx), r_sigma = interp(t->r_sigma, idx, didx);
  double n_eff = interp(t->n_eff, idx, didx);
  if (z > 10.) {
    return pow(D1, 4) * 2. *
           (F2_tree(k1, k2, k3) * linear_pk(t, k1) * linear_pk(t, k2) +
            F2_tree(k2, k3, k1) * linear_pk(t, k2) * linear_pk(t, k3) +
            F2_tree(k3, k1, k2) * linear_pk(t, k3) * linear_pk(t, k1));
  }
  double q[4];
  q[1] = k1 * r_sigma, q[2] = k2 * r_sigma, q[3] = k3 * r_sigma;
  for (int i = 1; i <= 3; i++)
    for (int j = i + 1; j <= 3; j++)
      if (q[i] < q[j]) std::swap(q[i], q[j]);
  double r1 = q[3] / q[1], r2 = (q[2] + q[3] - q[1]) / q[1];
  q[1] = k1 * r_sigma, q[2] = k2 * r_sigma, q[3] = k3 * r_sigma;
  double ls = log10(D1 * c.sigma8);
  double an = pow(10., -2.167 - 2.944 * ls - 1.106 * pow(ls, 2) - 2.865 * pow(ls, 3) -
                           0.310 * pow(r1, pow(10., 0.182 + 0.57 * n_eff)));
  double bn = pow(10., -3.428 - 2.681 * ls + 1.624 * pow(ls, 2) - 0.095 * pow(ls, 3));
  double cn = pow(10., 0.159 - 1.107 * n_eff);
  double alphan = pow(10., -4.348 - 3.006 * n_eff - 0.5745 * pow(n_eff, 2) + pow(10., -0.9 + 0.2 * n_eff) * pow(r2, 2));
  if (alphan > 1. - (2. / 3.) * c.ns) alphan = 1. - (2. / 3.) * c.ns;
  double betan = pow(10., -1.731 - 2.845 * n_eff - 1.4995 * pow(n_eff, 2) - 0.2811 * pow(n_eff, 3) + 0.007 * r2);
  double BS1h = 1.;
  for (int i = 1; i <= 3; i++) BS1h *= 1. / (an * pow(q[i], alphan) + bn * pow(q[i], betan)) / (1. + 1. / (cn * q[i]));
  double fn = pow(10., -10.533 - 16.838 * n_eff - 9.3048 * pow(n_eff, 2) - 1.8263 * pow(n_eff, 3));
  double gn = pow(10., 2.787 + 2.405 * n_eff + 0.4577 * pow(n_eff, 2));
  double hn = pow(10., -1.118 - 0.394 * n_eff);
  double mn = pow(10., -2.605 - 2.434 * ls + 5.71 * pow(ls, 2));
  double nn = pow(10., -4.468 - 3.08 * ls + 1.035 * pow(ls, 2));
  double mun = pow(10., 15.312 + 22.977 * n_eff + 10.9579 * pow(n_eff, 2) + 1.6586 * pow(n_eff, 3));
  double nun = pow(10., 1.347 + 1.246 * n_eff + 0.4525 * pow(n_eff, 2));
  double pn = pow(10., 0.071 - 0.433 * n_eff);
  double en = pow(10., -0.632 + 0.646 * n_eff);
  double PSE[4];
  for (int i = 1; i <= 3; i++)
    PSE[i] = (1. + fn * pow(q[i], 2)) / (1. + gn * q[i] + hn * pow(q[i], 2)) * pow(D1, 2) * linear_pk(t, q[i] / r_sigma) +
             1. / (mn * pow(q[i], mun) + nn * pow(q[i], nun)) / (1. + pow(pn * q[i], -3));
  double BS3h = 2. * (F2(t, k1, k2, k3, z, D1, r_sigma) * PSE[1] * PSE[2] + F2(t, k2, k3, k1, z, D1, r_sigma) * PSE[2] * PSE[3] +
                      F2(t, k3, k1, k2, z, D1, r_sigma) * PSE[3] * PSE[1]);
  for (int i = 1; i <= 3; i++) BS3h *= 1. / (1. + en * q[i]);
  return BS1h + BS3h;
}

// analytic Gaussian test bispectrum, classed_version/bispectrum.cpp:989-996
double bispectrum_analytic_single_a(double l1, double l2, double phi, double a) {
  double bis_pref = -pow(PI, 2) / (8 * 72 * pow(a, 8));
  double pref = pow(l1, 2) * pow(l2, 2) * (pow(l1, 2) + pow(l2, 2) + 2 * l1 * l2 * cos(phi));
  double expon = exp(-(pow(l1, 2) + pow(l2, 2) + l1 * l2 * cos(phi)) / (6 * a));
  return bis_pref * pref * expon;
}
const double AN_W[9] = {0, 1.0e+8, 1.0e+6, 1.0e+4, 1.0e+2, 1.0e+0, 5.0e-3, 1.0e-5, 1.0e-6};
const double AN_A[9] = {3.0e+3, 1.0e+4, 3.0e+4, 1.0e+5, 3.0e+5, 1.0e+6, 3.0e+6, 1.0e+7, 3.0e+7};

// LOS integrand of b_kappa, bispectrum.cu:311-333 (analytic mode:
// classed_version/bispectrum.cpp:477-499)
double integrand_bkappa(const orc_tables* t, double z, double l1, double l2, double l3) {
  if (t->analytic) {
    if (z > 1) return 0;
    double phi = PI - acos((l1 * l1 + l2 * l2 - l3 * l3) / (2 * l1 * l2));
    if (std::isnan(phi)) phi = 0;
    double temp = 0;
    for (int i = 0; i < 9; i++) temp += AN_W[i] * bispectrum_analytic_single_a(l1, l2, phi, AN_A[i]);
    temp /= (27. / 8. * pow(t->c.om, 3) * pow(100. / 299792., 5));
    return temp * 3.;
  }
  if (z < 1.0e-7) return 0.;
  if (l1 <= 1.0e-10 || l2 <= 1.0e-10 || l3 <= 1.0e-10) return 0;
  double didx = z / t->z_max * NZ;
  int idx = (int)didx;
  didx = didx - idx;
  clamp_idx(idx, didx);
  double g = interp(t->g, idx, didx), fK = interp(t->f_K, idx, didx);
  double r = pow(g * (1. + z), 3) * bispec(t, l1 / fK, l2 / fK, l3 / fK, z, idx, didx) / fK / E(t, z);
  if (std::isnan(r)) return 0;
  return r;
}

// bispectrum.cu:293-309
double bkappa(const orc_tables* t, double l1, double l2, double l3) {
  if (l1 == 0 || l2 == 0 || l3 == 0) return 0;
  double prefactor = 27. / 8. * pow(t->c.om, 3) * pow(H0_OVER_C, 5);
  const GQ96& G = gq96();
  double a = 0, b = t->z_max, cx = (a + b) / 2, dx = (b - a) / 2, q = 0;
  for (int i = 0; i < 48; i++)
    q += G.w[i] * (integrand_bkappa(t, cx - dx * G.a[i], l1, l2, l3) + integrand_bkappa(t, cx + dx * G.a[i], l1, l2, l3));
  return prefactor * (q * dx);
}

// P_kappa LOS integrand with the T17 correction, bispectrum.cu:951-991
double limber_integrand_power_spectrum(const orc_tables* t, double ell, double z) {
  if (z < 1e-5) return 0;
  double didx = z / t->z_max * (NZ - 1);
  int idx = (int)didx;
  didx = didx - idx;
  clamp_idx(idx, didx);
  double g = interp(t->g, idx, didx), fK = interp(t->f_K, idx, didx);
  double pref = 9. / 4. * H0_OVER_C * H0_OVER_C * H0_OVER_C * t->c.om * t->c.om * (1. + z) * (1. + z) * g * g / E(t, z);
  double k = ell / fK;
  const double c1 = 9.5171e-4, c2 = 5.1543e-3, a1 = 1.3063, a2 = 1.1475, a3 = 0.62793;
  double corr = pow(1 + c1 * pow(k, -1. * a1), a1) / pow(1 + c2 * pow(k, -1. * a2), a3);
  return corr * pref * P_k_nonlinear(t, ell / fK, z);
}

// device Pell = GQ96 LOS of P_kappa + shape noise, bispectrum.cu:511-529,935-949
double Pell(const orc_tables* t, double ell) {
  double P_sn = 0.5 * t->sigma * t->sigma / t->ngal;
  if (t->constant_ps) return P_sn;
  const GQ96& G = gq96();
  double a = 0, b = t->z_max, cx = (a + b) / 2, dx = (b - a) / 2, q = 0;
  for (int i = 0; i < 48; i++)
    q += G.w[i] * (limber_integrand_power_spectrum(t, ell, cx - dx * G.a[i]) +
                   limber_integrand_power_spectrum(t, ell, cx + dx * G.a[i]));
  return q * dx + P_sn;
}

// apertureStatistics.cu:18-22
double uHat(double eta) {
  double temp = 0.5 * eta * eta;
  return temp * exp(-temp);
}

}  // namespace

// ===========================================================================
// cubature: restatement of the reference's Gladwell-parallel hcubature_v
// ===========================================================================
namespace {

thread_local long g_last_neval = 0;

struct Region {
  std::vector<double> d;  // center[dim], halfwidth[dim]
  double vol = 0;
  unsigned splitDim = 0;
  std::vector<double> val, err;
  double errmax = HUGE_VAL;
};

double region_vol(const std::vector<double>& d, unsigned dim) {
  double v = 1;
  for (unsigned i = 0; i < dim; ++i) v *= 2 * d[i + dim];
  return v;
}

// hcubature.cpp:229-241 (halves: lower keeps the scaled volume, upper recomputes it)
void cut_region(Region& R, Region& R2, unsigned dim) {
  unsigned d = R.splitDim;
  R2 = R;
  R.d[d + dim] *= 0.5;
  R.vol *= 0.5;
  R2.d = R.d;
  R2.vol = region_vol(R2.d, dim);
  R.d[d] -= R.d[d + dim];
  R2.d[d] += R.d[d + dim];
}

struct Rule {
  unsigned dim, fdim, npts;
  std::vector<double> pts, vals;
  // Genz-Malik weights, hcubature.cpp:456-617
  double w1, w3, w5, wE1, wE3;
};

unsigned ls0(unsigned n) {
  unsigned b = 0;
  while (n & 1u) {
    n >>= 1;
    ++b;
  }
  return b;
}

const double GM_L2 = (double)sqrtl(9.0L / 70.0L);
const double GM_L4 = (double)sqrtl(9.0L / 10.0L);
const double GM_L5 = (double)sqrtl(9.0L / 19.0L);
const double GM_W2 = 980. / 6561., GM_W4 = 200. / 19683., GM_WE2 = 245. / 486., GM_WE4 = 25. / 729.;

void gm_points(const Region& R, unsigned dim, double* pts) {
  const double* c = R.d.data();
  const double* hw = R.d.data() + dim;
  std::vector<double> p(c, c + dim);
  size_t n = 0;
  auto store = [&]() { std::memcpy(pts + n * dim, p.data(), sizeof(double) * dim); ++n; };
  std::vector<double> r1(dim), r2(dim), r5(dim);
  for (unsigned i = 0; i < dim; ++i) {
    r1[i] = hw[i] * GM_L2;
    r2[i] = hw[i] * GM_L4;
    r5[i] = hw[i] * GM_L5;
  }
  store();  // center
  for (unsigned i = 0; i < dim; ++i) {
    p[i] = c[i] - r1[i]; store();
    p[i] = c[i] + r1[i]; store();
    p[i] = c[i] - r2[i]; store();
    p[i] = c[i] + r2[i]; store();
    p[i] = c[i];
  }
  for (unsigned i = 0; i + 1 < dim; ++i) {
    p[i] = c[i] - r2[i];
    for (unsigned j = i + 1; j < dim; ++j) {
      p[j] = c[j] - r2[j]; store();
      p[i] = c[i] + r2[i]; store();
      p[j] = c[j] + r2[j]; store();
      p[i] = c[i] - r2[i]; store();
      p[j] = c[j];
    }
    p[i] = c[i];
  }
  // 2^dim corners in Gray-code order starting from all "+"
  for (unsigned i = 0; i < dim; ++i) p[i] = c[i] + r5[i];
  unsigned signs = 0;
  for (unsigned i = 0;; ++i) {
    store();
    unsigned d = ls0(i);
    if (d >= dim) break;
    unsigned mask = 1u << d;
    signs ^= mask;
    p[d] = (signs & mask) ? c[d] - r5[d] : c[d] + r5[d];
  }
}

int eval_gm(Rule& r, orc_integrand_v f, void* fdata, std::vector<Region*>& Rs) {
  unsigned dim = r.dim, fdim = r.fdim;
  size_t nR = Rs.size();
  r.pts.resize(nR * r.npts * dim);
  r.vals.resize(nR * r.npts * fdim);
  for (size_t iR = 0; iR < nR; ++iR) gm_points(*Rs[iR], dim, r.pts.data() + iR * r.npts * dim);
  if (f(dim, nR * r.npts, r.pts.data(), fdata, fdim, r.vals.data())) return 1;
  const double ratio = (GM_L2 * GM_L2) / (GM_L4 * GM_L4);
  std::vector<double> diff(nR * dim, 0.0);
  for (unsigned j = 0; j < fdim; ++j) {
    const double* v = r.vals.data() + j;
    for (size_t iR = 0; iR < nR; ++iR) {
      auto V = [&](size_t i) { return v[fdim * i]; };
      double sum2 = 0, sum3 = 0, sum4 = 0, sum5 = 0;
      double val0 = V(0);
      unsigned k0 = 1, k;
      for (k = 0; k < dim; ++k) {
        double v0 = V(k0 + 4 * k), v1 = V(k0 + 4 * k + 1), v2 = V(k0 + 4 * k + 2), v3 = V(k0 + 4 * k + 3);
        sum2 += v0 + v1;
        sum3 += v2 + v3;
        diff[iR * dim + k] += fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
      }
      k0 += 4 * k;
      unsigned nrr = 2 * dim * (dim - 1);
      for (k = 0; k < nrr; ++k) sum4 += V(k0 + k);
      k0 += k;
      for (k = 0; k < (1u << dim); ++k) sum5 += V(k0 + k);
      Region& R = *Rs[iR];
      double result = R.vol * (r.w1 * val0 + GM_W2 * sum2 + r.w3 * sum3 + GM_W4 * sum4 + r.w5 * sum5);
      double res5th = R.vol * (r.wE1 * val0 + GM_WE2 * sum2 + r.wE3 * sum3 + GM_WE4 * sum4);
      R.val[j] = result;
      R.err[j] = fabs(res5th - result);
      v += r.npts * fdim;
    }
  }
  for (size_t iR = 0; iR < nR; ++iR) {
    double maxdiff = 0;
    unsigned dm = 0;
    for (unsigned i = 0; i < dim; ++i)
      if (diff[iR * dim + i] > maxdiff) {
        maxdiff = diff[iR * dim + i];
        dm = i;
      }
    Rs[iR]->splitDim = dm;
  }
  return 0;
}

// 15-point Gauss-Kronrod (QUADPACK constants), hcubature.cpp:620-780
const double GK_XGK[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                          0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                          0.586087235467691130294144838258730, 0.405845151377397166906606412076961,
                          0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
const double GK_WG[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                         0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
const double GK_WGK[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                          0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                          0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                          0.204432940075298892414161999234649, 0.209482141084727828012999174891714};

int eval_gk15(Rule& r, orc_integrand_v f, void* fdata, std::vector<Region*>& Rs) {
  unsigned fdim = r.fdim;
  size_t nR = Rs.size();
  r.pts.resize(nR * 15);
  r.vals.resize(nR * 15 * fdim);
  size_t np = 0;
  for (size_t iR = 0; iR < nR; ++iR) {
    double c = Rs[iR]->d[0], hw = Rs[iR]->d[1];
    r.pts[np++] = c;
    for (int j = 0; j < 3; ++j) {
      double w = hw * GK_XGK[2 * j + 1];
      r.pts[np++] = c - w;
      r.pts[np++] = c + w;
    }
    for (int j = 0; j < 4; ++j) {
      double w = hw * GK_XGK[2 * j];
      r.pts[np++] = c - w;
      r.pts[np++] = c + w;
    }
    Rs[iR]->splitDim = 0;
  }
  if (f(1, np, r.pts.data(), fdata, fdim, r.vals.data())) return 1;
  for (unsigned k = 0; k < fdim; ++k) {
    const double* vk = r.vals.data() + k;
    for (size_t iR = 0; iR < nR; ++iR) {
      double hw = Rs[iR]->d[1];
      double rg = vk[0] * GK_WG[3], rk = vk[0] * GK_WGK[7];
      double rabs = fabs(rk);
      size_t n = 1;
      for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        double v = vk[fdim * n] + vk[fdim * n + fdim];
        rg += GK_WG[j] * v;
        rk += GK_WGK[j2] * v;
        rabs += GK_WGK[j2] * (fabs(vk[fdim * n]) + fabs(vk[fdim * n + fdim]));
        n += 2;
      }
      for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rk += GK_WGK[j2] * (vk[fdim * n] + vk[fdim * n + fdim]);
        rabs += GK_WGK[j2] * (fabs(vk[fdim * n]) + fabs(vk[fdim * n + fdim]));
        n += 2;
      }
      Rs[iR]->val[k] = rk * hw;
      double mean = rk * 0.5;
      double rasc = GK_WGK[7] * fabs(vk[0] - mean);
      n = 1;
      for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        rasc += GK_WGK[j2] * (fabs(vk[fdim * n] - mean) + fabs(vk[fdim * n + fdim] - mean));
        n += 2;
      }
      for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rasc += GK_WGK[j2] * (fabs(vk[fdim * n] - mean) + fabs(vk[fdim * n + fdim] - mean));
        n += 2;
      }
      double e = fabs(rk - rg) * hw;
      rabs *= hw;
      rasc *= hw;
      if (rasc != 0 && e != 0) {
        double scale = pow((200 * e / rasc), 1.5);
        e = (scale < 1) ? rasc * scale : rasc;
      }
      if (rabs > DBL_MIN / (50 * DBL_EPSILON)) {
        double min_err = 50 * DBL_EPSILON * rabs;
        if (min_err > e) e = min_err;
      }
      Rs[iR]->err[k] = e;
      vk += 15 * fdim;
    }
  }
  return 0;
}

// converged.h
bool converged(unsigned fdim, const double* val, const double* err, double reqAbs, double reqRel, int norm) {
  switch (norm) {
    case ORC_ERROR_INDIVIDUAL:
      for (unsigned j = 0; j < fdim; ++j)
        if (err[j] > reqAbs && err[j] > fabs(val[j]) * reqRel) return false;
      return true;
    case ORC_ERROR_PAIRED: {
      unsigned j;
      for (j = 0; j + 1 < fdim; j += 2) {
        double maxerr = err[j] > err[j + 1] ? err[j] : err[j + 1];
        double maxval = val[j] > val[j + 1] ? val[j] : val[j + 1];
        double serr = maxerr > 0 ? 1 / maxerr : 1, sval = maxval > 0 ? 1 / maxval : 1;
        double e = sqrt((err[j] * serr) * (err[j] * serr) + (err[j + 1] * serr) * (err[j + 1] * serr)) * maxerr;
        double v = sqrt((val[j] * sval) * (val[j] * sval) + (val[j + 1] * sval) * (val[j + 1] * sval)) * maxval;
        if (e > reqAbs && e > v * reqRel) return false;
      }
      if (j < fdim)
        if (err[j] > reqAbs && err[j] > fabs(val[j]) * reqRel) return false;
      return true;
    }
    case ORC_ERROR_L1: {
      double e = 0, v = 0;
      for (unsigned j = 0; j < fdim; ++j) {
        e += err[j];
        v += fabs(val[j]);
      }
      return e <= reqAbs || e <= v * reqRel;
    }
    case ORC_ERROR_LINF: {
      double e = 0, v = 0;
      for (unsigned j = 0; j < fdim; ++j) {
        double a = fabs(val[j]);
        if (err[j] > e) e = err[j];
        if (a > v) v = a;
      }
      return e <= reqAbs || e <= v * reqRel;
    }
    case ORC_ERROR_L2: {
      double maxerr = 0, maxval = 0, e = 0, v = 0;
      for (unsigned j = 0; j < fdim; ++j) {
        double a = fabs(val[j]);
        if (err[j] > maxerr) maxerr = err[j];
        if (a > maxval) maxval = a;
      }
      double serr = maxerr > 0 ? 1 / maxerr : 1, sval = maxval > 0 ? 1 / maxval : 1;
      for (unsigned j = 0; j < fdim; ++j) {
        e += (err[j] * serr) * (err[j] * serr);
        v += (fabs(val[j]) * sval) * (fabs(val[j]) * sval);
      }
      e = sqrt(e) * maxerr;
      v = sqrt(v) * maxval;
      return e <= reqAbs || e <= v * reqRel;
    }
  }
  return true;
}

// binary max-heap keyed on errmax with running totals (hcubature.cpp:790-900)
struct Heap {
  std::vector<Region> items;
  size_t n = 0;
  std::vector<double> tv, te;
  explicit Heap(unsigned fdim) : tv(fdim, 0.0), te(fdim, 0.0) {}
  void push(const Region& hi) {
    for (size_t i = 0; i < tv.size(); ++i) {
      tv[i] += hi.val[i];
      te[i] += hi.err[i];
    }
    size_t ins = n;
    if (++n > items.size()) items.resize(n * 2);
    while (ins) {
      size_t parent = (ins - 1) / 2;
      if (hi.errmax <= items[parent].errmax) break;
      items[ins] = items[parent];
      ins = parent;
    }
    items[ins] = hi;
  }
  Region pop() {
    Region ret = items[0];
    size_t i = 0, m = --n;
    items[0] = items[m];
    size_t child;
    while ((child = i * 2 + 1) < m) {
      size_t largest = (items[child].errmax <= items[i].errmax) ? i : child;
      if (++child < m && items[largest].errmax < items[child].errmax) largest = child;
      if (largest == i) break;
      std::swap(items[i], items[largest]);
      i = largest;
    }
    for (size_t k = 0; k < tv.size(); ++k) {
      tv[k] -= ret.val[k];
      te[k] -= ret.err[k];
    }
    return ret;
  }
};

}  // namespace

extern "C" int orc_hcubature_v(unsigned fdim, orc_integrand_v f, void* fdata, unsigned dim,
                               const double* xmin, const double* xmax, size_t maxEval, double reqAbs,
                               double reqRel, int norm, double* val, double* err) {
  g_last_neval = 0;
  if (fdim == 0) return 0;
  if (dim == 0) {
    if (f(0, 1, xmin, fdata, fdim, val)) return 1;
    for (unsigned i = 0; i < fdim; ++i) err[i] = 0;
    return 0;
  }
  if (fdim <= 1) norm = ORC_ERROR_INDIVIDUAL;
  if (norm < 0 || norm > ORC_ERROR_LINF) return 1;
  Rule r;
  r.dim = dim;
  r.fdim = fdim;
  if (dim == 1) {
    r.npts = 15;
  } else {
    if (dim >= 32) return 1;
    r.npts = 1 + 2 * 2 * dim + 2 * dim * (dim - 1) + (1u << dim);
    int d = (int)dim;
    r.w1 = (double)(12824 - 9120 * d + 400 * d * d) / 19683.0;
    r.w3 = (double)(1820 - 400 * d) / 19683.0;
    r.w5 = 6859.0 / 19683.0 / (double)(1u << dim);
    r.wE1 = (double)(729 - 950 * d + 50 * d * d) / 729.0;
    r.wE3 = (double)(265 - 100 * d) / 1458.0;
  }
  auto eval = [&](std::vector<Region*>& Rs) -> int {
    int rc = dim == 1 ? eval_gk15(r, f, fdata, Rs) : eval_gm(r, f, fdata, Rs);
    if (rc) return rc;
    for (Region* R : Rs) {
      double m = 0;
      for (unsigned k = 0; k < fdim; ++k)
        if (R->err[k] > m) m = R->err[k];
      R->errmax = m;
    }
    return 0;
  };
  Region R0;
  R0.d.resize(2 * dim);
  for (unsigned i = 0; i < dim; ++i) {
    R0.d[i] = 0.5 * (xmin[i] + xmax[i]);
    R0.d[i + dim] = 0.5 * (xmax[i] - xmin[i]);
  }
  R0.vol = region_vol(R0.d, dim);
  R0.val.assign(fdim, 0.0);
  R0.err.assign(fdim, 0.0);
  Heap heap(fdim);
  size_t numEval = 0;
  {
    std::vector<Region*> Rs{&R0};
    if (eval(Rs)) return 1;
    heap.push(R0);
    numEval += r.npts;
  }
  std::vector<Region> R;
  std::vector<double> ee(fdim), ev(fdim);
  while (numEval < maxEval || !maxEval) {
    if (converged(fdim, heap.tv.data(), heap.te.data(), reqAbs, reqRel, norm)) break;
    R.clear();
    ee = heap.te;
    ev = heap.tv;
    do {
      R.push_back(heap.pop());
      for (unsigned j = 0; j < fdim; ++j) ee[j] -= R.back().err[j];
      R.emplace_back();
      cut_region(R[R.size() - 2], R.back(), dim);
      numEval += r.npts * 2;
      if (converged(fdim, ev.data(), ee.data(), reqAbs, reqRel, norm)) break;
    } while (heap.n > 0 && (numEval < maxEval || !maxEval));
    std::vector<Region*> Rs;
    for (auto& x : R) Rs.push_back(&x);
    if (eval(Rs)) return 1;
    for (auto& x : R) heap.push(x);
  }
  for (unsigned j = 0; j < fdim; ++j) val[j] = err[j] = 0;
  for (size_t i = 0; i < heap.n; ++i)
    for (unsigned j = 0; j < fdim; ++j) {
      val[j] += heap.items[i].val[j];
      err[j] += heap.items[i].err[j];
    }
  g_last_neval = (long)numEval;
  return 0;
}

extern "C" long orc_last_neval(void) { return g_last_neval; }

// ===========================================================================
// tables and scalar wrappers
// ===========================================================================
extern "C" orc_tables* orc_tables_create(const orc_cosmo* c, const double* nz, const double* pk, double dk,
                                         double kmin, double kmax) {
  orc_tables* t = new orc_tables();
  t->c = *c;
  // set_cosmology, bispectrum.cu:148-212. With a given P(k) the reference
  // still builds norm, r_sigma, n_eff and ncur from Eisenstein & Hu: its
  // set_cosmology declares a local `bool Pk_given` (bispectrum.cu:132) that
  // shadows the global flag the host linear_pk reads (:36, :623), and the
  // host Pk/dk/k_min/k_max globals are never filled. Only the device-side
  // linear_pk (dev_Pk_given, :605-621) reads the table. So the table is
  // attached after the build.
  t->norm = 1;
  t->norm = t->c.sigma8 / sigmam(t, 8., 0);
  t->z_max = t->c.zmax;
  t->dz = t->z_max / NZ;
  const double dz = t->dz;
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < NZ; i++) t->f_K[i] = f_K_at_z(t, (i + 0.5) * dz);
  for (int i = 0; i < NZ; i++) {
    double gi = 0;
    for (int j = i; j < NZ; j++) {
      double term = nz[j] * (t->f_K[j] - t->f_K[i]) / t->f_K[j];
      gi += (j == i || j == NZ - 1) ? term / 2 : term;
    }
    t->g[i] = gi * dz;
  }
  t->g[0] = 1.;
  double lgr0 = lgr(t, 0.);
#pragma omp parallel for schedule(dynamic)
  for (int i = 0; i < NZ; i++) {
    double z = (i + 0.5) * dz;
    t->D1[i] = lgr(t, z) / lgr0;
    t->r_sigma[i] = calc_r_sigma(t, t->D1[i]);
    double s2 = sigmam(t, t->r_sigma[i], 2);
    double d1 = -2. * pow(t->D1[i] * s2, 2);
    t->n_eff[i] = -3. + 2. * pow(t->D1[i] * s2, 2);
    t->ncur[i] = d1 * d1 + 4. * sigmam(t, t->r_sigma[i], 3) * pow(t->D1[i], 2);
  }
  if (pk) {
    t->pk_given = true;
    std::memcpy(t->pk, pk, sizeof(double) * NK);
    t->dk = dk;
    t->kmin = kmin;
    t->kmax = kmax;
  }
  return t;
}

extern "C" void orc_tables_destroy(orc_tables* t) { delete t; }
extern "C" void orc_tables_get(const orc_tables* t, double* out) {
  std::memcpy(out + 0 * NZ, t->f_K, sizeof(double) * NZ);
  std::memcpy(out + 1 * NZ, t->g, sizeof(double) * NZ);
  std::memcpy(out + 2 * NZ, t->D1, sizeof(double) * NZ);
  std::memcpy(out + 3 * NZ, t->r_sigma, sizeof(double) * NZ);
  std::memcpy(out + 4 * NZ, t->n_eff, sizeof(double) * NZ);
  std::memcpy(out + 5 * NZ, t->ncur, sizeof(double) * NZ);
  out[6 * NZ] = t->norm;
}
extern "C" void orc_set_noise(orc_tables* t, double sigma, double ngal, int constant_ps) {
  t->sigma = sigma;
  t->ngal = ngal;
  t->constant_ps = constant_ps != 0;
}
extern "C" void orc_set_analytic(orc_tables* t, int on) { t->analytic = on != 0; }

extern "C" double orc_E(const orc_tables* t, double z) { return E(t, z); }
extern "C" double orc_linear_pk(const orc_tables* t, double k) { return linear_pk(t, k); }
extern "C" double orc_sigmam(const orc_tables* t, double r, int j) { return sigmam(t, r, j); }
extern "C" double orc_lgr(const orc_tables* t, double z) { return lgr(t, z); }
extern "C" double orc_calc_r_sigma(const orc_tables* t, double D1) { return calc_r_sigma(t, D1); }
extern "C" double orc_f_K_at_z(const orc_tables* t, double z) { return f_K_at_z(t, z); }
extern "C" double orc_P_k_nonlinear(const orc_tables* t, double k, double z) { return P_k_nonlinear(t, k, z); }
extern "C" double orc_bispec_at_z(const orc_tables* t, double k1, double k2, double k3, double z) {
  double didx = z / t->z_max * NZ;
  int idx = (int)didx;
  didx -= idx;
  clamp_idx(idx, didx);
  return bispec(t, k1, k2, k3, z, idx, didx);
}
extern "C" double orc_integrand_bkappa(const orc_tables* t, double z, double l1, double l2, double l3) {
  return integrand_bkappa(t, z, l1, l2, l3);
}
extern "C" double orc_bkappa(const orc_tables* t, double l1, double l2, double l3) { return bkappa(t, l1, l2, l3); }
extern "C" void orc_bkappa_batch(const orc_tables* t, const double* ell, long n, double* out) {
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < n; ++i) out[i] = bkappa(t, ell[3 * i], ell[3 * i + 1], ell[3 * i + 2]);
}
extern "C" double orc_Pell(const orc_tables* t, double ell) { return Pell(t, ell); }
extern "C" double orc_limber_integrand(const orc_tables* t, double ell, double z) {
  return limber_integrand_power_spectrum(t, ell, z);
}
extern "C" double orc_uHat(double eta) { return uHat(eta); }
extern "C" void orc_gq96(double* a, double* w) {
  std::memcpy(a, gq96().a, sizeof(double) * 48);
  std::memcpy(w, gq96().w, sizeof(double) * 48);
}
extern "C" void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n <= 0) n = omp_get_num_procs();
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// ===========================================================================
// <Map^3>
// ===========================================================================
struct orc_map3_ctx {
  const orc_tables* t;
  double th[3];
};
extern "C" orc_map3_ctx* orc_map3_ctx_create(const orc_tables* t, double a, double b, double c) {
  return new orc_map3_ctx{t, {a, b, c}};
}
extern "C" void orc_map3_ctx_destroy(orc_map3_ctx* c) { delete c; }

// integrand_Map3_kernel, apertureStatistics.cu:138-153
extern "C" int orc_integrand_map3_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned fdim,
                                    double* fval) {
  (void)fdim;
  const orc_map3_ctx* m = (const orc_map3_ctx*)fdata;
#pragma omp parallel for schedule(dynamic, 4) if (npts > 64)
  for (long i = 0; i < (long)npts; ++i) {
    double l1 = x[i * ndim], l2 = x[i * ndim + 1], phi = x[i * ndim + 2];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
    fval[i] = l1 * l2 * bkappa(m->t, l1, l2, l3) * uHat(l1 * m->th[0]) * uHat(l2 * m->th[1]) * uHat(l3 * m->th[2]);
  }
  return 0;
}

// MapMapMap, apertureStatistics.cu:201-230
extern "C" double orc_MapMapMap(const orc_tables* t, const double* th, double phiMin, double phiMax, double lMin,
                                double lMax, double relTol, double* err, long* neval) {
  double thetaMin = std::min({th[0], th[1], th[2]});
  if (lMax <= 0) lMax = 10. / thetaMin;
  orc_map3_ctx ctx{t, {th[0], th[1], th[2]}};
  double xmin[3] = {lMin, lMin, phiMin}, xmax[3] = {lMax, lMax, phiMax};
  double res = 0, e = 0;
  orc_hcubature_v(1, orc_integrand_map3_v, &ctx, 3, xmin, xmax, 0, 0, relTol, ORC_ERROR_L1, &res, &e);
  const double norm = 1. / 8 / PI / PI / PI;
  if (err) *err = e * norm;
  if (neval) *neval = orc_last_neval();
  return res * norm;
}

// ===========================================================================
// shear 3PCF
// ===========================================================================
namespace {

// zeros of J_nu by Newton iteration from McMahon's asymptotic expansion
double bessel_zero(int nu, int s) {
  if (s == 0) return 0.0;
  double mu = 4.0 * nu * nu;
  double b = (s + 0.5 * nu - 0.25) * PI;
  double x = b - (mu - 1) / (8 * b) - 4 * (mu - 1) * (7 * mu - 31) / (3 * pow(8 * b, 3));
  if (s == 1) {  // small-s guesses from the asymptotic form are poor for large nu
    x = nu + 1.8557571 * pow((double)nu, 1.0 / 3.0) + 1.033150 * pow((double)nu, -1.0 / 3.0);
    if (nu == 0) x = 2.404825557695773;
  }
  for (int it = 0; it < 100; ++it) {
    double J = std::cyl_bessel_j((double)nu, x);
    double dJ = 0.5 * (std::cyl_bessel_j((double)nu - 1, x) - std::cyl_bessel_j((double)nu + 1, x));
    double dx = J / dJ;
    x -= dx;
    if (fabs(dx) < 1e-15 * x) break;
  }
  return x;
}
double psi_fn(double t) { return t * tanh(PI * sinh(t) / 2); }
double psip_fn(double t) {
  double num = sinh(PI * sinh(t)) + PI * t * cosh(t);
  double den = cosh(PI * sinh(t)) + 1;
  return num / den;
}
// Ogata step and node count: the CUDA values by default (gamma.cuh:29-30:
// prec_h = 0.1, prec_k = int(3.31 / 0.1)); orc_set_ogata changes them (the
// classed test of the analytic bispectrum uses h = 0.01, k up to 3.5).
double g_prec_h = 0.1;
int g_prec_k = 33;

struct Ogata {
  double h = 0;
  int nk = 0;
  std::vector<double> psi6, prod6, psi2, prod2;
  void build(double hh, int n) {
    h = hh;
    nk = n;
    psi6.assign(n, 0), prod6.assign(n, 0), psi2.assign(n, 0), prod2.assign(n, 0);
    // compute_weights_bessel, gamma.cu:13-56
    for (int pass = 0; pass < 2; ++pass) {
      int nu = pass == 0 ? 6 : 2;
      double* ps = pass == 0 ? psi6.data() : psi2.data();
      double* pr = pass == 0 ? prod6.data() : prod2.data();
      for (int i = 0; i < n; ++i) {
        double z = bessel_zero(nu, i);
        double pz = z / PI;
        ps[i] = PI * psi_fn(pz * h) / h;
        double Jb = std::cyl_bessel_j((double)nu, ps[i]);
        double pp = psip_fn(h * pz);
        double Jn1 = i == 0 ? 0.0 : std::cyl_bessel_j((double)nu + 1, z);
        double w = 2 / (PI * z * pow(Jn1, 2));
        pr[i] = w * pow(ps[i], 3) * Jb * pp;
      }
    }
  }
};
const Ogata& ogata() {
  static Ogata o;
  if (o.h != g_prec_h || o.nk != g_prec_k) o.build(g_prec_h, g_prec_k);
  return o;
}

typedef std::complex<double> cplx;

// triangle geometry, gamma.cu:491-529
double interior_angle(double an1, double an2, double opp) {
  return acos((pow(an1, 2) + pow(an2, 2) - pow(opp, 2)) / (2.0 * an1 * an2));
}
double A_fn(double psi, double x1, double x2, double phi, double varpsi) {
  return sqrt(pow(cos(psi) * x2, 2) + pow(sin(psi) * x1, 2) + sin(2 * psi) * x1 * x2 * cos(phi + varpsi));
}
double alpha_fn(double psi, double x1, double x2, double phi, double varpsi) {
  double num = (cos(psi) * x2 - sin(psi) * x1) * sin((phi + varpsi) / 2);
  double den = (cos(psi) * x2 + sin(psi) * x1) * cos((phi + varpsi) / 2);
  return atan2(num, den);
}
double betabar(double psi, double phi) {
  double num = cos(2 * psi) * sin(phi);
  double den = cos(phi) + sin(2 * psi);
  return 0.5 * atan2(num, den);
}
cplx exp_of_imag(double x) { return cplx(cos(x), sin(x)); }
cplx prefactor(double x1, double x2, double x3, double phi, double psi) {
  double varpsi = interior_angle(x1, x2, x3);
  cplx e = exp_of_imag(interior_angle(x2, x3, x1) - interior_angle(x1, x3, x2) - 6 * alpha_fn(psi, x1, x2, phi, varpsi));
  cplx pphi = exp_of_imag(2. * betabar(psi, phi));
  return e * pphi * sin(2 * psi);
}

// gamma.cu:463-482
cplx one_integrand_gamma0(const orc_tables* t, double phi, double psi, double z, int k, double x1, double x2, double x3) {
  const Ogata& O = ogata();
  double varpsi = interior_angle(x1, x2, x3);
  double A3 = A_fn(psi, x1, x2, phi, varpsi);
  cplx pre = prefactor(x1, x2, x3, phi, psi);
  double ell1 = O.psi6[k] / A3 * cos(psi);
  double ell2 = O.psi6[k] / A3 * sin(psi);
  double ell3 = ell1 * ell1 + ell2 * ell2 + 2 * ell1 * ell2 * cos(phi);
  ell3 = ell3 <= 0 ? 0 : sqrt(ell3);
  double bis = integrand_bkappa(t, z, ell1, ell2, ell3) * O.prod6[k] * PI / pow(A3, 4);
  return pre * bis;
}
cplx full_integrand_gamma0(const orc_tables* t, double phi, double psi, double z, int k, double x1, double x2, double x3) {
  return (one_integrand_gamma0(t, phi, psi, z, k, x1, x2, x3) + one_integrand_gamma0(t, phi, psi, z, k, x2, x3, x1)) +
         one_integrand_gamma0(t, phi, psi, z, k, x3, x1, x2);
}
// gamma.cu:419-456
cplx full_integrand_gamma1(const orc_tables* t, double phi, double psi, double z, int k, double x1, double x2, double x3) {
  const Ogata& O = ogata();
  double vb = betabar(psi, phi);
  double p1 = interior_angle(x2, x3, x1), p2 = interior_angle(x3, x1, x2), p3 = interior_angle(x1, x2, x3);
  double A1 = A_fn(psi, x2, x3, phi, p1), A2 = A_fn(psi, x3, x1, phi, p2), A3 = A_fn(psi, x1, x2, phi, p3);
  double al1 = alpha_fn(psi, x2, x3, phi, p1), al2 = alpha_fn(psi, x3, x1, phi, p2), al3 = alpha_fn(psi, x1, x2, phi, p3);
  double ell1 = O.psi2[k] * cos(psi), ell2 = O.psi2[k] * sin(psi);
  double ell3 = ell1 * ell1 + ell2 * ell2 + 2 * ell1 * ell2 * cos(phi);
  ell3 = ell3 <= 0 ? 0 : sqrt(ell3);
  cplx i3 = exp_of_imag(p1 - p2 + 2 * p3 + 2 * (vb - phi - al3)) *
            (integrand_bkappa(t, z, ell1 / A3, ell2 / A3, ell3 / A3) * PI / pow(A3, 4));
  cplx i1 = exp_of_imag(p3 - p2 - 2 * (vb + al1)) * (integrand_bkappa(t, z, ell1 / A1, ell2 / A1, ell3 / A1) * PI / pow(A1, 4));
  cplx i2 = exp_of_imag(p3 - p1 - 2 * p2 + 2 * (vb + phi - al2)) *
            (integrand_bkappa(t, z, ell1 / A2, ell2 / A2, ell3 / A2) * PI / pow(A2, 4));
  return (i1 + (i2 + i3)) * (sin(2 * psi) * O.prod2[k]);
}

struct GammaCtx {
  const orc_tables* t;
  int which;  // 0 -> Gamma0 integrand, 1 -> Gamma1 integrand
  double x1, x2, x3;
};
int integrand_gamma_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned fdim, double* fval) {
  (void)ndim;
  (void)fdim;
  const GammaCtx* g = (const GammaCtx*)fdata;
#pragma omp parallel for schedule(dynamic, 4) if (npts > 64)
  for (long i = 0; i < (long)npts; ++i) {
    double z = x[i * 3], phi = x[i * 3 + 1], psi = x[i * 3 + 2];
    const int nk = ogata().nk;
    cplx s0(0, 0);
    if (nk == 33) {
      // pairwise tree over k=1..32 as the shared-memory reduction (gamma.cu:291-305)
      cplx v[32];
      for (int k = 1; k < nk; ++k)
        v[k - 1] = g->which == 0 ? full_integrand_gamma0(g->t, phi, psi, z, k, g->x1, g->x2, g->x3)
                                 : full_integrand_gamma1(g->t, phi, psi, z, k, g->x1, g->x2, g->x3);
      for (int size = 16; size > 0; size /= 2)
        for (int j = 0; j < size; ++j) v[j] += v[j + size];
      s0 = v[0];
    } else {
      for (int k = 1; k < nk; ++k)
        s0 += g->which == 0 ? full_integrand_gamma0(g->t, phi, psi, z, k, g->x1, g->x2, g->x3)
                            : full_integrand_gamma1(g->t, phi, psi, z, k, g->x1, g->x2, g->x3);
    }
    fval[2 * i] = s0.real();
    fval[2 * i + 1] = s0.imag();
  }
  return 0;
}

// gamma.cu:72-96
double height_of_triangle(double x1, double x2, double x3) { return 0.5 * sqrt(2 * pow(x1, 2) + 2 * pow(x2, 2) - pow(x3, 2)); }
double one_rotation_angle_otc(double x1, double x2, double x3) {
  double psi3 = interior_angle(x1, x2, x3);
  double h3 = height_of_triangle(x1, x2, x3);
  double c2 = pow(pow(x2, 2) - pow(x1, 2), 2) - 4 * pow(x1 * x2 * sin(psi3), 2);
  c2 /= pow(2 * h3 * x3, 2);
  double s2 = (pow(x2, 2) - pow(x1, 2)) * x1 * x2 * sin(psi3);
  s2 /= pow(h3 * x3, 2);
  return atan2(s2, c2) / 2;
}
cplx orthocenter_to_centroid(cplx g, double x1, double x2, double x3, bool conj1) {
  double a1 = one_rotation_angle_otc(x2, x3, x1);
  double a2 = one_rotation_angle_otc(x3, x1, x2);
  double a3 = one_rotation_angle_otc(x1, x2, x3);
  if (conj1) a1 *= -1.;
  return g * std::exp(cplx(0, -2.) * (a1 + a2 + a3));
}

}  // namespace

extern "C" void orc_set_ogata(double h, int nk) {
  g_prec_h = h;
  g_prec_k = nk;
  (void)ogata();  // build now, outside any parallel region
}

extern "C" void orc_ogata_weights(double* out) {
  const Ogata& O = ogata();
  const int n = O.nk;
  for (int k = 0; k < n; ++k) {
    out[k] = O.psi6[k];
    out[n + k] = O.prod6[k];
    out[2 * n + k] = O.psi2[k];
    out[3 * n + k] = O.prod2[k];
  }
}

// gamma0..gamma3, gamma.cu:98-148
extern "C" void orc_gamma(const orc_tables* t, int comp, double x1, double x2, double x3, double relTol,
                          double absTol, double* re, double* im, long* neval) {
  (void)ogata();  // the node table is built on the calling thread
  if (comp == 2) {  // gamma2 = gamma1(x2,x3,x1)
    orc_gamma(t, 1, x2, x3, x1, relTol, absTol, re, im, neval);
    return;
  }
  if (comp == 3) {  // gamma3 = gamma1(x3,x1,x2)
    orc_gamma(t, 1, x3, x1, x2, relTol, absTol, re, im, neval);
    return;
  }
  GammaCtx g{t, comp, x1, x2, x3};
  double xmin[3] = {0, 0, 0}, xmax[3] = {t->z_max, 2 * PI, PI / 2};
  double res[2], err[2];
  orc_hcubature_v(2, integrand_gamma_v, &g, 3, xmin, xmax, 0, absTol, relTol, ORC_ERROR_L1, res, err);
  if (neval) *neval = orc_last_neval();
  cplx r(res[0], res[1]);
  r = orthocenter_to_centroid(r, x1, x2, x3, comp == 1);
  r = r * 27. / 8. * pow(t->c.om, 3) * pow(100. / 299792., 5) / 3. / (2 * pow(2 * PI, 3));
  *re = r.real();
  *im = r.imag();
}

// The Gamma cubature integrand at given points (z, phi, psi): the sum over the
// Ogata nodes k = 1 .. prec_k-1 of full_integrand_gamma0 (which = 0) or
// full_integrand_gamma1 (which = 1), as compute_integrand_gamma0/1 form it
// per point (gamma.cu:267-363); out[2i], out[2i+1] = real, imaginary part.
extern "C" void orc_gamma_integrand_points(const orc_tables* t, int which, double x1, double x2, double x3,
                                           const double* pts, long n, double* out) {
  (void)ogata();
  GammaCtx g{t, which, x1, x2, x3};
  integrand_gamma_v(3, (size_t)n, pts, &g, 2, out);
}

// closed-form Gamma^0 for the analytic test bispectrum,
// classed_version/gamma.cpp:83-93,567-582
extern "C" void orc_ggg_analytic(double r1, double r2, double r3, double* re, double* im) {
  cplx tot(0, 0);
  for (int i = 0; i < 9; ++i) {
    double a = AN_A[i];
    cplx x(r2, 0);
    double height = (r1 + r2 + r3) * (r2 + r3 - r1) * (r1 - r2 + r3) * (r1 + r2 - r3);
    height = sqrt(height) / (2. * r2);
    double rest = sqrt(r1 * r1 - height * height);
    cplx y(-rest, -height);
    cplx z = -x - y;
    double phi1 = atan2(imag(x), real(x)), phi2 = atan2(imag(y), real(y)), phi3 = atan2(imag(z), real(z));
    cplx pref = std::pow((x + 2. * y) * (x - y) * (y + 2. * x), 2);
    double expon = std::norm(x) + std::norm(y) + real(x) * real(y) + imag(x) * imag(y);
    cplx phase = std::exp(cplx(0, -2.) * (phi1 + phi2 + phi3));
    tot += AN_W[i] * (pref * exp(-2 * a * expon) * phase);
  }
  *re = tot.real();
  *im = tot.imag();
}

// ===========================================================================
// <Map^3> covariance: T1 (square / infinite), T2 (square), T4 (infinite)
// ===========================================================================
namespace {

// window of a square survey, apertureStatisticsCovariance.cu:132-153, and of
// a rectangle with sides thetaMax (x) and thetaMaxY (y), :154-172
double G_rect(double thetaMax, double thetaMaxY, double lx, double ly) {
  double t1 = 0.5 * lx * thetaMax, t2 = 0.5 * ly * thetaMaxY;
  double j1 = fabs(t1) <= 1e-6 ? 1 : sin(t1) / t1;
  double j2 = fabs(t2) <= 1e-6 ? 1 : sin(t2) / t2;
  return j1 * j1 * j2 * j2;
}
// circular window, apertureStatisticsCovariance.cu:117-130
double G_square(double thetaMax, double lx, double ly) { return G_rect(thetaMax, thetaMax, lx, ly); }
// second side of the window: thetaMax except for the rectangle
double side_y(const orc_cov_params* p) { return p->type == 3 ? p->thetaMaxSmaller : p->thetaMax; }
double G_circle(double thetaMax, double ell) {
  double tmp = thetaMax * ell;
  double r = std::cyl_bessel_j(1.0, tmp);
  r *= r;
  r *= 4 / tmp / tmp;
  return r;
}

struct CovCtx {
  const orc_tables* t;
  const orc_cov_params* p;
  double th[6];
  double lMax;
};

// integrand_T1_square / _infinite / _circle, apertureStatisticsCovariance.cu:1886-1982
int integrand_T1_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const CovCtx* c = (const CovCtx*)fdata;
  const double* th = c->th;
#pragma omp parallel for schedule(dynamic, 4) if (npts > 64)
  for (long i = 0; i < (long)npts; ++i) {
    const double* v = x + i * ndim;
    double res = 0;
    if (c->p->type == 2) {
      double l1 = v[0], l2 = v[1], phi = v[2];
      double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
      double lmin = c->p->lMin;
      if (!(l1 <= lmin || l2 <= lmin || l3 <= lmin || l3 > c->lMax)) {
        res = Pell(c->t, l1) * Pell(c->t, l2) * Pell(c->t, l3);
        res *= uHat(l1 * th[0]) * uHat(l2 * th[1]) * uHat(l3 * th[2]);
        res *= uHat(l1 * th[3]) * uHat(l2 * th[4]) * uHat(l3 * th[5]);
        res *= l1 * l2;
      }
    } else {
      double a = v[0], b = v[1], cc = v[2], d = v[3], e = v[4], f = v[5];
      double ell1 = sqrt((a - cc - e) * (a - cc - e) + (b - d - f) * (b - d - f));
      double ell2 = sqrt(cc * cc + d * d);
      double ell3 = sqrt(e * e + f * f);
      bool zero;
      double G;
      if (c->p->type == 1 || c->p->type == 3) {
        G = G_rect(c->p->thetaMax, side_y(c->p), a, b);
        zero = ell1 <= 0 || ell2 <= 0 || ell3 <= 0 || ell3 > c->lMax;
      } else {
        G = G_circle(c->p->thetaMax, sqrt(a * a + b * b));
        double lmin = c->p->lMin;
        zero = ell1 <= lmin || ell2 <= lmin || ell3 <= lmin;
      }
      if (!zero) {
        res = Pell(c->t, ell1) * Pell(c->t, ell2) * Pell(c->t, ell3);
        res *= uHat(ell1 * th[0]) * uHat(ell2 * th[1]) * uHat(ell3 * th[2]);
        res *= uHat(ell1 * th[3]) * uHat(ell2 * th[4]) * uHat(ell3 * th[5]);
        res *= G;
      }
    }
    fval[i] = res;
  }
  return 0;
}

// integrand_T2_part1 / _part2_square, apertureStatisticsCovariance.cu:2019-2089
struct T2Ctx {
  const orc_tables* t;
  const orc_cov_params* p;
  double th1, th2;
  int part;  // 1 or 2
};
int integrand_T2_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const T2Ctx* c = (const T2Ctx*)fdata;
  for (long i = 0; i < (long)npts; ++i) {
    double res = 0;
    if (c->part == 1) {
      double ell = x[i * ndim];
      if (!(ell < c->p->lMin)) res = ell * Pell(c->t, ell) * uHat(ell * c->th1) * uHat(ell * c->th2);
    } else if (c->p->type == 1 || c->p->type == 3) {
      double lx = x[i * ndim], ly = x[i * ndim + 1];
      double G = G_rect(c->p->thetaMax, side_y(c->p), lx, ly);
      double ell = sqrt(lx * lx + ly * ly);
      // ell = 0 (the centre of the symmetric box) is the integrand's limit 0;
      // the reference evaluates Pell(0) there, which is NaN
      if (!(ell < c->p->lMin) && ell > 0) res = Pell(c->t, ell) * uHat(ell * c->th1) * uHat(ell * c->th2) * G;
    } else {  // circle
      double ell = x[i * ndim];
      if (!(ell < c->p->lMin))
        res = Pell(c->t, ell) * ell * uHat(ell * c->th1) * uHat(ell * c->th2) * G_circle(c->p->thetaMax, ell);
    }
    fval[i] = res;
  }
  return 0;
}

// integrand_T4_infinite, apertureStatisticsCovariance.cu:2118-2149
int integrand_T4_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const CovCtx* c = (const CovCtx*)fdata;
  const double* th = c->th;
#pragma omp parallel for schedule(dynamic, 2) if (npts > 16)
  for (long i = 0; i < (long)npts; ++i) {
    const double* v = x + i * ndim;
    double l1 = exp(v[0]), l2 = exp(v[1]), l5 = exp(v[2]), phi1 = v[3], phi2 = v[4];
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi1));
    double l6 = sqrt(l1 * l1 + l5 * l5 + 2 * l1 * l5 * cos(phi2));
    double res = 0;
    if (!(l3 > c->lMax || l6 > c->lMax || l3 <= 0 || l6 <= 0)) {
      res = uHat(l1 * th[0]) * uHat(l2 * th[1]) * uHat(l3 * th[2]) * uHat(l1 * th[3]) * uHat(l5 * th[4]) * uHat(l6 * th[5]);
      res *= bkappa(c->t, l1, l2, l3);
      res *= bkappa(c->t, l1, l5, l6);
      res *= l1 * l2 * l5;
      res *= l1 * l2 * l5;
    }
    fval[i] = res;
  }
  return 0;
}

}  // namespace

extern "C" double orc_G_square(double thetaMax, double lx, double ly) { return G_square(thetaMax, lx, ly); }

// T1, apertureStatisticsCovariance.cu:1065-1106
extern "C" double orc_T1(const orc_tables* t, const orc_cov_params* p, const double* th, double relTol, long* neval) {
  double tmin123 = std::min({th[0], th[1], th[2]}), tmin456 = std::min({th[3], th[4], th[5]});
  double lMax = 10. / std::max(tmin123, tmin456);
  CovCtx c{t, p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  double res = 0, err = 0;
  if (p->type == 2) {
    double xmin[3] = {p->lMin, p->lMin, 0}, xmax[3] = {lMax, lMax, PI};
    orc_hcubature_v(1, integrand_T1_v, &c, 3, xmin, xmax, 0, 0, relTol > 0 ? relTol : 1e-4, ORC_ERROR_L1, &res, &err);
    res *= 2 / p->area / pow(2 * PI, 3);
  } else {
    double xmin[6], xmax[6];
    for (int i = 0; i < 6; ++i) {
      xmin[i] = -lMax;
      xmax[i] = 1.02 * lMax;
    }
    orc_hcubature_v(1, integrand_T1_v, &c, 6, xmin, xmax, 0, 0, relTol > 0 ? relTol : 1e-2, ORC_ERROR_L1, &res, &err);
    res /= pow(2 * PI, 6);
  }
  if (neval) *neval = orc_last_neval();
  return res;
}

// The 6-D finite-field T1 of orc_T1 with an evaluation cap (maxEval, the
// hcubature_v argument the reference passes as 0 = unbounded): the value and
// error estimate reached after about maxEval integrand points, to measure how
// far a configuration's integral is from the requested tolerance.
extern "C" double orc_T1_capped(const orc_tables* t, const orc_cov_params* p, const double* th, double relTol,
                                long maxEval, double* err_out, long* neval) {
  double tmin123 = std::min({th[0], th[1], th[2]}), tmin456 = std::min({th[3], th[4], th[5]});
  double lMax = 10. / std::max(tmin123, tmin456);
  CovCtx c{t, p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  double xmin[6], xmax[6], res = 0, err = 0;
  for (int i = 0; i < 6; ++i) {
    xmin[i] = -lMax;
    xmax[i] = 1.02 * lMax;
  }
  orc_hcubature_v(1, integrand_T1_v, &c, 6, xmin, xmax, (size_t)maxEval, 0, relTol > 0 ? relTol : 1e-2, ORC_ERROR_L1,
                  &res, &err);
  if (neval) *neval = orc_last_neval();
  if (err_out) *err_out = err / pow(2 * PI, 6);
  return res / pow(2 * PI, 6);
}

// T2, apertureStatisticsCovariance.cu:1108-1164 (the 1-D upper bound is the
// one computed from theta1..theta5 and is reused for the second 1-D integral)
extern "C" double orc_T2(const orc_tables* t, const orc_cov_params* p, const double* th) {
  if (p->type == 2) return 0;
  double thetaMin = std::min({th[0], th[1], th[2], th[3], th[4]});
  double lMax = 10. / thetaMin;
  double vmin1[1] = {p->lMin}, vmax1[1] = {lMax};
  double rA1, eA1, rA2, eA2, rB, eB;
  T2Ctx c{t, p, th[0], th[1], 1};
  orc_hcubature_v(1, integrand_T2_v, &c, 1, vmin1, vmax1, 0, 0, 1e-4, ORC_ERROR_L1, &rA1, &eA1);
  rA1 /= 2 * PI;
  c.th1 = th[4];
  c.th2 = th[5];
  orc_hcubature_v(1, integrand_T2_v, &c, 1, vmin1, vmax1, 0, 0, 1e-4, ORC_ERROR_L1, &rA2, &eA2);
  rA2 /= 2 * PI;
  c.th1 = th[2];
  c.th2 = th[3];
  c.part = 2;
  lMax = 10. / std::min(th[2], th[3]);
  if (p->type == 0) {
    orc_hcubature_v(1, integrand_T2_v, &c, 1, vmin1, vmax1, 0, 0, 1e-4, ORC_ERROR_L1, &rB, &eB);
    rB /= 2 * PI;
  } else {
    double vmin2[2] = {-lMax, -lMax}, vmax2[2] = {lMax, lMax};
    orc_hcubature_v(1, integrand_T2_v, &c, 2, vmin2, vmax2, 0, 0, 1e-4, ORC_ERROR_L1, &rB, &eB);
    rB /= pow(2 * PI, 2);
  }
  return rA1 * rA2 * rB;
}

// T4, apertureStatisticsCovariance.cu:1166-1197 (infinite geometry only)
extern "C" double orc_T4(const orc_tables* t, const orc_cov_params* p, const double* th, double relTol, long* neval) {
  double tmin123 = std::min({th[0], th[1], th[2]}), tmin456 = std::min({th[3], th[4], th[5]});
  double lMax = 10. / std::max(tmin123, tmin456);
  double lMin = 1e-5;
  CovCtx c{t, p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  double xmin[5] = {log(lMin), log(lMin), log(lMin), 0, 0};
  double xmax[5] = {log(lMax), log(lMax), log(lMax), 2 * PI, 2 * PI};
  double res = 0, err = 0;
  orc_hcubature_v(1, integrand_T4_v, &c, 5, xmin, xmax, 0, 0, relTol > 0 ? relTol : 1e-2, ORC_ERROR_L1, &res, &err);
  if (neval) *neval = orc_last_neval();
  return res / p->area / pow(2 * PI, 5);
}

// permutation tables of T1_total / T2_total / T4_total are shared with the
// product through tests only; the oracle evaluates them directly here.
namespace {
typedef double (*TermFn)(const orc_tables*, const orc_cov_params*, const double*);
double t1fn(const orc_tables* t, const orc_cov_params* p, const double* th) { return orc_T1(t, p, th, 0, nullptr); }
double t2fn(const orc_tables* t, const orc_cov_params* p, const double* th) { return orc_T2(t, p, th); }
double t4fn(const orc_tables* t, const orc_cov_params* p, const double* th) { return orc_T4(t, p, th, 0, nullptr); }
double call(TermFn f, const orc_tables* t, const orc_cov_params* p, double a, double b, double c, double d, double e, double g) {
  double th[6] = {a, b, c, d, e, g};
  return f(t, p, th);
}
}  // namespace

// T1_total, apertureStatisticsCovariance.cu:272-326
static double T1_total_with(TermFn f, const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  double t0 = A[0], t1 = A[1], t2 = A[2], t3 = B[0], t4 = B[1], t5 = B[2];
  double r;
  if (t3 == t4) {
    if (t4 == t5)
      r = 6 * call(f, t, p, t0, t1, t2, t3, t3, t3);
    else
      r = 2 * call(f, t, p, t0, t1, t2, t3, t3, t5) + 2 * call(f, t, p, t0, t1, t2, t3, t5, t3) +
          2 * call(f, t, p, t0, t1, t2, t5, t3, t3);
  } else if (t3 == t5) {
    r = 2 * call(f, t, p, t0, t1, t2, t3, t4, t3) + 2 * call(f, t, p, t0, t1, t2, t3, t3, t4) +
        2 * call(f, t, p, t0, t1, t2, t4, t3, t3);
  } else if (t4 == t5) {
    r = 2 * call(f, t, p, t0, t1, t2, t3, t4, t4) + 2 * call(f, t, p, t0, t1, t2, t4, t3, t4) +
        2 * call(f, t, p, t0, t1, t2, t4, t4, t3);
  } else {
    r = call(f, t, p, t0, t1, t2, t3, t4, t5) + call(f, t, p, t0, t1, t2, t3, t5, t4) +
        call(f, t, p, t0, t1, t2, t4, t3, t5) + call(f, t, p, t0, t1, t2, t4, t5, t3) +
        call(f, t, p, t0, t1, t2, t5, t3, t4) + call(f, t, p, t0, t1, t2, t5, t4, t3);
  }
  return r;
}

// T2_total, apertureStatisticsCovariance.cu:328-538
static double T2_total_with(TermFn f, const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  if (p->type == 2) return 0;
  double a0 = A[0], a1 = A[1], a2 = A[2], b0 = B[0], b1 = B[1], b2 = B[2];
  auto T = [&](double x0, double x1, double x2, double y0, double y1, double y2) { return call(f, t, p, x0, x1, x2, y0, y1, y2); };
  double r;
  // the nine first-triplet cases of the reference, written as (multiplicity, args)
  if (a0 == a1 && a1 == a2) {
    if (b0 == b1 && b1 == b2) r = 9 * T(a0, a0, a0, b0, b0, b0);
    else if (b0 == b1) r = 6 * T(a0, a0, a0, b0, b0, b2) + 3 * T(a0, a0, a0, b2, b0, b0);
    else if (b0 == b2) r = 6 * T(a0, a0, a0, b0, b1, b0) + 3 * T(a0, a0, a0, b1, b0, b0);
    else if (b1 == b2) r = 6 * T(a0, a0, a0, b1, b0, b1) + 3 * T(a0, a0, a0, b0, b1, b1);
    else r = 3 * T(a0, a0, a0, b0, b1, b2) + 3 * T(a0, a0, a0, b1, b0, b2) + 3 * T(a0, a0, a0, b2, b0, b1);
  } else if (a0 == a1) {
    if (b0 == b1 && b1 == b2) r = 6 * T(a0, a2, a0, b0, b0, b0) + 3 * T(a0, a0, a2, b0, b0, b0);
    else if (b0 == b1) r = 2 * T(a0, a0, a2, b0, b0, b2) + T(a0, a0, a2, b2, b0, b0) + 4 * T(a0, a2, a0, b0, b0, b2) + 2 * T(a0, a2, a0, b2, b0, b0);
    else if (b0 == b2) r = 2 * T(a0, a0, a2, b0, b1, b0) + T(a0, a0, a2, b1, b0, b0) + 4 * T(a0, a2, a0, b0, b1, b0) + 2 * T(a0, a2, a0, b1, b0, b0);
    else if (b1 == b2) r = 2 * T(a0, a0, a2, b1, b0, b1) + T(a0, a0, a2, b0, b1, b1) + 4 * T(a0, a2, a0, b1, b0, b1) + 2 * T(a0, a2, a0, b0, b1, b1);
    else r = T(a0, a0, a2, b0, b1, b2) + T(a0, a0, a2, b1, b0, b2) + T(a0, a0, a2, b2, b0, b1) + 2 * T(a0, a2, a0, b0, b1, b2) + 2 * T(a0, a2, a0, b1, b0, b2) + 2 * T(a0, a2, a0, b2, b0, b1);
  } else if (a1 == a2) {
    if (b0 == b1 && b1 == b2) r = 6 * T(a0, a1, a1, b0, b0, b0) + 3 * T(a1, a1, a0, b0, b0, b0);
    else if (b0 == b1) r = 2 * T(a0, a1, a1, b2, b0, b0) + T(a1, a1, a0, b2, b0, b0) + 4 * T(a0, a1, a1, b0, b0, b2) + 2 * T(a1, a1, a0, b0, b0, b2);
    else if (b0 == b2) r = 4 * T(a0, a1, a1, b0, b1, b0) + 2 * T(a0, a1, a1, b1, b0, b0) + 2 * T(a1, a1, a0, b0, b1, b0) + T(a1, a1, a0, b1, b0, b0);
    else if (b1 == b2) r = 2 * T(a0, a1, a1, b0, b1, b1) + T(a1, a1, a0, b0, b1, b1) + 4 * T(a0, a1, a1, b1, b0, b1) + 2 * T(a1, a1, a0, b1, b0, b1);
    else r = 2 * T(a0, a1, a1, b0, b1, b2) + 2 * T(a0, a1, a1, b1, b0, b2) + 2 * T(a0, a1, a1, b2, b0, b1) + T(a1, a1, a0, b0, b1, b2) + T(a1, a1, a0, b1, b0, b2) + T(a1, a1, a0, b2, b0, b1);
  } else if (a0 == a2) {
    if (b0 == b1 && b1 == b2) r = 6 * T(a0, a1, a0, b0, b0, b0) + 3 * T(a1, a0, a0, b0, b0, b0);
    else if (b0 == b1) r = 2 * T(a0, a1, a0, b2, b0, b0) + T(a1, a0, a0, b2, b0, b0) + 4 * T(a0, a1, a0, b0, b0, b2) + 2 * T(a1, a0, a0, b0, b0, b2);
    else if (b0 == b2) r = 4 * T(a0, a1, a0, b0, b1, b0) + 2 * T(a0, a1, a0, b1, b0, b0) + 2 * T(a1, a0, a0, b0, b1, b0) + T(a1, a0, a0, b1, b0, b0);
    else if (b1 == b2) r = 2 * T(a0, a1, a0, b0, b1, b1) + T(a1, a0, a0, b0, b1, b1) + 4 * T(a0, a1, a0, b1, b0, b1) + 2 * T(a1, a0, a0, b1, b0, b1);
    else r = 2 * T(a0, a1, a0, b0, b1, b2) + 2 * T(a0, a1, a0, b1, b0, b2) + 2 * T(a0, a1, a0, b2, b0, b1) + T(a1, a0, a0, b0, b1, b2) + T(a1, a0, a0, b1, b0, b2) + T(a1, a0, a0, b2, b0, b1);
  } else {
    if (b0 == b1 && b1 == b2) r = 3 * T(a0, a1, a2, b0, b0, b0) + 3 * T(a0, a2, a1, b0, b0, b0) + 3 * T(a1, a2, a0, b0, b0, b0);
    else if (b0 == b1) r = 2 * T(a0, a1, a2, b0, b0, b2) + T(a0, a1, a2, b2, b0, b0) + 2 * T(a0, a2, a1, b0, b0, b2) + T(a0, a2, a1, b2, b0, b0) + 2 * T(a1, a2, a0, b0, b0, b2) + T(a1, a2, a0, b2, b0, b0);
    else if (b0 == b2) r = 2 * T(a0, a1, a2, b0, b1, b0) + T(a0, a1, a2, b1, b0, b0) + 2 * T(a0, a2, a1, b0, b1, b0) + T(a0, a2, a1, b1, b0, b0) + 2 * T(a1, a2, a0, b0, b1, b0) + T(a1, a2, a0, b1, b0, b0);
    else if (b1 == b2) r = 2 * T(a0, a1, a2, b1, b0, b1) + T(a0, a1, a2, b0, b1, b1) + 2 * T(a0, a2, a1, b1, b0, b1) + T(a0, a2, a1, b0, b1, b1) + 2 * T(a1, a2, a0, b1, b0, b1) + T(a1, a2, a0, b0, b1, b1);
    else r = T(a0, a1, a2, b0, b1, b2) + T(a0, a1, a2, b1, b0, b2) + T(a0, a1, a2, b2, b0, b1) + T(a0, a2, a1, b0, b1, b2) + T(a0, a2, a1, b1, b0, b2) + T(a0, a2, a1, b2, b0, b1) + T(a1, a2, a0, b0, b1, b2) + T(a1, a2, a0, b1, b0, b2) + T(a1, a2, a0, b2, b0, b1);
  }
  return r;
}

// T4_total, apertureStatisticsCovariance.cu:540-683 (argument patterns kept
// as the reference evaluates them, including its uneven th4==th5 branch)
static double T4_total_with(TermFn f, const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  double t0 = A[0], t1 = A[1], t2 = A[2], t3 = B[0], t4 = B[1], t5 = B[2];
  auto T = [&](double x0, double x1, double x2, double y0, double y1, double y2) { return call(f, t, p, x0, x1, x2, y0, y1, y2); };
  double r;
  if (t0 == t1 && t0 == t2) {
    if (t3 == t4 && t3 == t5) r = 9 * T(t3, t0, t0, t0, t3, t3);
    else if (t3 == t4) r = 6 * T(t3, t0, t0, t0, t3, t5) + 3 * T(t5, t0, t0, t0, t3, t3);
    else r = 3 * T(t3, t0, t0, t0, t4, t5) + 3 * T(t4, t0, t0, t0, t3, t5) + 3 * T(t5, t0, t0, t0, t3, t4);
  } else if (t0 == t1) {
    if (t3 == t4 && t3 == t5) r = 6 * T(t3, t0, t2, t0, t3, t3) + 3 * T(t3, t0, t0, t2, t3, t3);
    else if (t3 == t4) r = 2 * T(t3, t0, t0, t2, t3, t5) + 4 * T(t3, t0, t2, t0, t3, t5) + T(t5, t0, t0, t2, t3, t3) + 2 * T(t5, t0, t2, t0, t3, t3);
    else r = T(t3, t0, t0, t2, t4, t5) + 2 * T(t3, t0, t2, t0, t4, t5) + T(t4, t0, t0, t2, t3, t5) + 2 * T(t4, t0, t2, t0, t3, t5) + T(t5, t0, t0, t2, t3, t4) + 2 * T(t5, t0, t2, t0, t3, t4);
  } else if (t3 == t4) {
    if (t3 == t5) r = 3 * T(t3, t0, t1, t2, t3, t3) + 3 * T(t3, t0, t2, t1, t3, t3) + 3 * T(t3, t1, t2, t0, t3, t3);
    else r = 2 * T(t3, t0, t1, t2, t3, t5) + 2 * T(t3, t0, t2, t1, t3, t5) + 2 * T(t3, t1, t2, t0, t3, t5) + T(t5, t0, t1, t2, t3, t4) + T(t5, t1, t2, t0, t3, t3) + T(t5, t0, t2, t1, t3, t3);
  } else if (t4 == t5) {
    r = T(t3, t0, t1, t2, t4, t5) + T(t3, t0, t2, t1, t4, t5) + T(t3, t1, t2, t0, t4, t4) + 2 * T(t4, t0, t1, t2, t3, t4) + 2 * T(t4, t1, t2, t0, t3, t4) + 2 * T(t4, t0, t2, t1, t3, t4);
  } else {
    r = T(t3, t0, t1, t2, t4, t5) + T(t3, t0, t2, t1, t4, t5) + T(t3, t1, t2, t0, t4, t5) + T(t4, t0, t1, t2, t3, t5) + T(t4, t0, t2, t1, t3, t5) + T(t4, t1, t2, t0, t3, t5) + T(t5, t0, t1, t2, t3, t4) + T(t5, t0, t2, t1, t3, t4) + T(t5, t1, t2, t0, t3, t4);
  }
  return r;
}

extern "C" double orc_T1_total(const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  return T1_total_with(t1fn, t, p, A, B);
}
extern "C" double orc_T2_total(const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  return T2_total_with(t2fn, t, p, A, B);
}
extern "C" double orc_T4_total(const orc_tables* t, const orc_cov_params* p, const double* A, const double* B) {
  return T4_total_with(t4fn, t, p, A, B);
}

// The totals of T1, T2, T4 with the term replaced by probe(th6): checks the
// argument patterns and multiplicities of another implementation of the
// totals without integrating anything (geometry 1 = square, 2 = infinite).
namespace {
double (*g_probe)(const double*) = nullptr;
double probe_fn(const orc_tables*, const orc_cov_params*, const double* th) { return g_probe(th); }
}  // namespace
extern "C" double orc_total_probe(int term, int geometry, double (*probe)(const double*), const double* A,
                                  const double* B) {
  g_probe = probe;
  orc_cov_params p{};
  p.type = geometry;
  if (term == 1) return T1_total_with(probe_fn, nullptr, &p, A, B);
  if (term == 2) return T2_total_with(probe_fn, nullptr, &p, A, B);
  return T4_total_with(probe_fn, nullptr, &p, A, B);
}

// ===========================================================================
// Halo model (cuda_version/halomodel.cu) and the covariance terms built on
// it: T5, T6, T7 (apertureStatisticsCovariance.cu:685-1063,1199-1313,2151-2314)
// ===========================================================================
namespace {

constexpr int NM = 128;                          // n_mbins, halomodel.cuh:17
constexpr double LOGMMIN = 9, LOGMMAX = 17;      // halomodel.cuh:15-16
constexpr double RHO_CRIT = 2.7754e11;           // [Msun h^2 / Mpc^3], halomodel.cu:54

// sigma^2(m) at z = 0: top-hat variance of radius R(m), adaptive 1-D
// integral over k in [0, 1e12] at relative 1e-4 (halomodel.cu:179-220)
struct SigmaCtx {
  const orc_tables* t;
  double R, dR;
  int deriv;
};
int integrand_sigma_v(unsigned ndim, size_t npts, const double* k, void* fdata, unsigned, double* fval) {
  const SigmaCtx* c = (const SigmaCtx*)fdata;
  for (size_t i = 0; i < npts; ++i) {
    double k_ = k[i * ndim];
    double W = window(k_ * c->R, 0);
    if (c->deriv)
      fval[i] = k_ * k_ * W * window(k_ * c->R, 4) * c->dR * linear_pk(c->t, k_) * k_;
    else
      fval[i] = k_ * k_ * W * W * linear_pk(c->t, k_);
  }
  return 0;
}

// setSigma2 / setdSigma2dm (halomodel.cu:197-214,262-276): masses
// m_i = 10^(logMmin + i (logMmax - logMmin) / n_mbins). The host linear_pk
// the reference calls there is always Eisenstein & Hu (its Pk_given global is
// never set; see orc_tables_create), so a given P(k) table is ignored here.
void ensure_halo(const orc_tables* tc) {
  orc_tables* t = const_cast<orc_tables*>(tc);
  if (t->halo) return;
  const bool given = t->pk_given;
  t->pk_given = false;
  const double rhobar = RHO_CRIT * t->c.om;
  const double deltaM = (LOGMMAX - LOGMMIN) / NM;
  for (int i = 0; i < NM; ++i) {
    double m = pow(10, LOGMMIN + i * deltaM);
    SigmaCtx c{t, pow(0.75 / PI * m / rhobar, 1. / 3.), 0, 0};
    double kmin[1] = {0}, kmax[1] = {1e12}, r, e;
    orc_hcubature_v(1, integrand_sigma_v, &c, 1, kmin, kmax, 0, 0, 1e-4, ORC_ERROR_L1, &r, &e);
    t->sig2[i] = r / 2 / PI / PI;
    c.dR = pow(0.75 / PI / rhobar, 1. / 3.) * pow(m, -2. / 3.) / 3.;
    c.deriv = 1;
    orc_hcubature_v(1, integrand_sigma_v, &c, 1, kmin, kmax, 0, 0, 1e-4, ORC_ERROR_L1, &r, &e);
    t->dsig2[i] = r / PI / PI;
  }
  t->pk_given = given;
  t->halo = true;
}

// linear interpolation in a z-table on the grid z_i = i z_max / (n - 1), as
// the halo-model code reads the tables (halomodel.cu:300-311,398-408), which
// set_cosmology fills at the bin centres (i + 0.5) z_max / n
double halo_zinterp(const orc_tables* t, const double* arr, double z) {
  double didx = z / t->z_max * (NZ - 1);
  int idx = (int)didx;
  didx = didx - idx;
  if (idx == NZ - 1) {
    idx = NZ - 2;
    didx = 1.;
  }
  return arr[idx] * (1 - didx) + arr[idx + 1] * didx;
}

// mass-table lookup, halomodel.cu:279-299: the index runs over n_mbins - 1
// intervals of [logMmin, logMmax] (the table was filled with n_mbins)
double halo_minterp(const double* arr, double m) {
  double didx = (log10(m) - LOGMMIN) / (LOGMMAX - LOGMMIN) * (NM - 1);
  int idx = (int)didx;
  didx = didx - idx;
  if (idx == NM - 1) {
    idx = NM - 2;
    didx = 1.;
  }
  return arr[idx] * (1 - didx) + arr[idx + 1] * didx;
}

// get_sigma2 / get_dSigma2dm, halomodel.cu:279-375
double get_sigma2(const orc_tables* t, double m, double z) {
  double D1 = halo_zinterp(t, t->D1, z);
  return halo_minterp(t->sig2, m) * D1 * D1;
}
double get_dsigma2(const orc_tables* t, double m, double z) {
  double D1 = halo_zinterp(t, t->D1, z);
  return halo_minterp(t->dsig2, m) * D1 * D1;
}

// Sheth-Tormen mass function dn/dm, halomodel.cu:31-59
double hmf(const orc_tables* t, double m, double z) {
  const double A = 0.322, q = 0.707, p = 0.3;
  double sigma2 = get_sigma2(t, m, z);
  double dsigma2 = get_dsigma2(t, m, z);
  double deltac = 1.686 * (1 + 0.0123 * log10(om_m_of_z(t, z)));
  double rho_mean = RHO_CRIT * t->c.om;
  double nu = deltac * deltac / sigma2;
  return -rho_mean / m / sigma2 * dsigma2 * A * (1 + pow(q * nu, -p)) * sqrt(q * nu / 2 / PI) * exp(-0.5 * q * nu);
}

// Sine and cosine integrals Si(x), Ci(x) by the rational approximations the
// reference uses (halomodel.cu:61-105; the Pade approximants of Rowe et al.
// 2015, GalSim, Appendix B: x < 4 a ratio of even polynomials, x >= 4 the
// auxiliary functions f, g in 1/x^2)
void sici(double x, double& si, double& ci) {
  double x2 = x * x, x4 = x2 * x2, x6 = x2 * x4, x8 = x4 * x4, x10 = x8 * x2, x12 = x6 * x6, x14 = x12 * x2;
  if (x < 4) {
    double a = 1 - 4.54393409816329991e-2 * x2 + 1.15457225751016682e-3 * x4 - 1.41018536821330254e-5 * x6 +
               9.43280809438713025e-8 * x8 - 3.53201978997168357e-10 * x10 + 7.08240282274875911e-13 * x12 -
               6.05338212010422477e-16 * x14;
    double b = 1 + 1.01162145739225565e-2 * x2 + 4.99175116169755106e-5 * x4 + 1.55654986308745614e-7 * x6 +
               3.28067571055789734e-10 * x8 + 4.5049097575386581e-13 * x10 + 3.21107051193712168e-16 * x12;
    si = x * a / b;
    a = -0.25 + 7.51851524438898291e-3 * x2 - 1.27528342240267686e-4 * x4 + 1.05297363846239184e-6 * x6 -
        4.68889508144848019e-9 * x8 + 1.06480802891189243e-11 * x10 - 9.93728488857585407e-15 * x12;
    b = 1 + 1.1592605689110735e-2 * x2 + 6.72126800814254432e-5 * x4 + 2.55533277086129636e-7 * x6 +
        6.97071295760958946e-10 * x8 + 1.38536352772778619e-12 * x10 + 1.89106054713059759e-15 * x12 +
        1.39759616731376855e-18 * x14;
    ci = 0.5772156649 + std::log(x) + x2 * a / b;
    return;
  }
  double x16 = x8 * x8, x18 = x16 * x2, x20 = x10 * x10;
  double cx = cos(x), sx = sin(x);
  double f = (1 + 7.44437068161936700618e2 / x2 + 1.96396372895146869801e5 / x4 + 2.37750310125431834034e7 / x6 +
              1.43073403821274636888e9 / x8 + 4.33736238870432522765e10 / x10 + 6.40533830574022022911e11 / x12 +
              4.20968180571076940208e12 / x14 + 1.00795182980368574617e13 / x16 + 4.94816688199951963482e12 / x18 -
              4.94701168645415959931e11 / x20) /
             (1 + 7.46437068161927678031e2 / x2 + 1.97865247031583951450e5 / x4 + 2.41535670165126845144e7 / x6 +
              1.47478952192985464958e9 / x8 + 4.58595115847765779830e10 / x10 + 7.08501308149515401563e11 / x12 +
              5.06084464593475076774e12 / x14 + 1.43468549171581016479e13 / x16 + 1.11535493509914254097e13 / x18) /
             x;
  double g = (1 + 8.1359520115168615e2 / x2 + 2.35239181626478200e5 / x4 + 3.12557570795778731e7 / x6 +
              2.06297595146763354e9 / x8 + 6.83052205423625007e10 / x10 + 1.09049528450362786e12 / x12 +
              7.57664583257834349e12 / x14 + 1.81004487464664575e13 / x16 + 6.43291613143049485e12 / x18 -
              1.36517137670871689e12 / x20) /
             (1 + 8.19595201151451564e2 / x2 + 2.40036752835578777e5 / x4 + 3.26026661647090822e7 / x6 +
              2.23355543278099360e9 / x8 + 7.87465017341829930e10 / x10 + 1.39866710696414565e12 / x12 +
              1.17164723371736605e13 / x14 + 4.01839087307656620e13 / x16 + 3.99653257887490811e13 / x18) /
             x2;
  si = 0.5 * PI - f * cx - g * sx;
  ci = f * sx - g * cx;
}

// halomodel.cu:107-119 (r_200 [Mpc/h]), :142-152 (Duffy et al. 2008 concentration)
double r_200(const orc_tables* t, double m) { return pow(0.75 / PI * m / (RHO_CRIT * t->c.om) / 200, 1. / 3.); }
double concentration(double m, double z) { return 10.14 * pow(m / 2e12, -0.081) * pow(1 + z, -1.01); }

// Fourier transform of the NFW profile truncated at r_200, halomodel.cu:121-140
double u_nfw(const orc_tables* t, double k, double m, double z) {
  double c = concentration(m, z);
  double arg1 = k * r_200(t, m) / c;
  double arg2 = arg1 * (1 + c);
  double si1, ci1, si2, ci2;
  sici(arg1, si1, ci1);
  sici(arg2, si2, ci2);
  double term1 = sin(arg1) * (si2 - si1);
  double term2 = cos(arg1) * (ci2 - ci1);
  double term3 = -sin(arg1 * c) / arg2;
  double F = std::log(1. + c) - c / (1. + c);
  return (term1 + term2 + term3) / F;
}

// one-halo convergence tri- and pentaspectrum integrands at (m, z) and their
// 96-point Gauss-Legendre line-of-sight integrals (halomodel.cu:392-510)
double trispectrum_integrand(const orc_tables* t, double m, double z, double l1, double l2, double l3, double l4) {
  double g = halo_zinterp(t, t->g, z);
  double chi = halo_zinterp(t, t->f_K, z);
  double rhobar = RHO_CRIT * t->c.om;
  double result = hmf(t, m, z) * g * g * g * g / chi / chi;
  result *= C_OVER_H0 / E(t, z);
  result *= u_nfw(t, l1 / chi, m, z) * u_nfw(t, l2 / chi, m, z) * u_nfw(t, l3 / chi, m, z) * u_nfw(t, l4 / chi, m, z);
  result *= m * m * m * m / rhobar / rhobar / rhobar / rhobar;
  result *= pow(1.5 * t->c.om / C_OVER_H0 / C_OVER_H0, 4);
  result *= pow(1 + z, 4);
  return result;
}
double trispectrum_los(const orc_tables* t, double m, double l1, double l2, double l3, double l4) {
  const GQ96& G = gq96();
  double cx = t->z_max / 2, dx = t->z_max / 2, q = 0;
  for (int i = 0; i < 48; i++)
    q += G.w[i] * (trispectrum_integrand(t, m, cx - dx * G.a[i], l1, l2, l3, l4) +
                   trispectrum_integrand(t, m, cx + dx * G.a[i], l1, l2, l3, l4));
  return q * dx;
}
double pentaspectrum_integrand(const orc_tables* t, double m, double z, const double* l) {
  double g = halo_zinterp(t, t->g, z);
  double chi = halo_zinterp(t, t->f_K, z);
  double rhobar = RHO_CRIT * t->c.om;
  double result = 1;
  result *= pow(g, 6);
  result /= pow(chi, 4);
  result *= C_OVER_H0 / E(t, z);
  result *= u_nfw(t, l[0] / chi, m, z) * u_nfw(t, l[1] / chi, m, z) * u_nfw(t, l[2] / chi, m, z);
  result *= u_nfw(t, l[3] / chi, m, z) * u_nfw(t, l[4] / chi, m, z) * u_nfw(t, l[5] / chi, m, z);
  result *= pow(m / rhobar, 6) * hmf(t, m, z);
  result *= pow(1.5 * t->c.om / C_OVER_H0 / C_OVER_H0, 6);
  result *= pow(1 + z, 6);
  return result;
}
double pentaspectrum_los(const orc_tables* t, double m, const double* l) {
  const GQ96& G = gq96();
  double cx = t->z_max / 2, dx = t->z_max / 2, q = 0;
  for (int i = 0; i < 48; i++)
    q += G.w[i] * (pentaspectrum_integrand(t, m, cx - dx * G.a[i], l) + pentaspectrum_integrand(t, m, cx + dx * G.a[i], l));
  return q * dx;
}

// integrand_T5_infinite, integrand_T6_square / _rectangle, integrand_T7_infinite
// (apertureStatisticsCovariance.cu:2151-2314). The reference's device lower
// bound dev_lMin is the driver's lMin = 0 (calculateApertureStatisticsCovariance.cu:89,
// uploaded once by initCovariance), so only l <= 0 is cut; a squared length
// that rounds below zero counts as zero length.
struct HaloCtx {
  const orc_tables* t;
  const orc_cov_params* p;
  double th[6];
  double lMax;
};
int integrand_T5_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const HaloCtx* c = (const HaloCtx*)fdata;
  const double* th = c->th;
#pragma omp parallel for schedule(dynamic, 1) if (npts > 8)
  for (long i = 0; i < (long)npts; ++i) {
    const double* v = x + i * ndim;
    double l1 = exp(v[0]), l2 = exp(v[1]), l5 = exp(v[2]), phi1 = v[3], phi2 = v[4], m = v[5];
    double s3 = l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi1);
    double s6 = l1 * l1 + l5 * l5 + 2 * l1 * l5 * cos(phi2);
    double res = 0;
    if (s3 > 0 && s6 > 0) {
      double l3 = sqrt(s3), l6 = sqrt(s6), l4 = l1;
      if (!(l3 > c->lMax || l6 > c->lMax)) {
        res = uHat(l1 * th[0]) * uHat(l2 * th[1]) * uHat(l3 * th[2]) * uHat(l4 * th[3]) * uHat(l5 * th[4]) *
              uHat(l6 * th[5]);
        res *= Pell(c->t, l1);
        res *= trispectrum_los(c->t, m, l2, l3, l5, l6);
        res *= l1 * l2 * l5;
        res *= l1 * l2 * l5;
      }
    }
    fval[i] = res;
  }
  return 0;
}
int integrand_T6_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const HaloCtx* c = (const HaloCtx*)fdata;
  const double* th = c->th;
#pragma omp parallel for schedule(dynamic, 1) if (npts > 8)
  for (long i = 0; i < (long)npts; ++i) {
    const double* v = x + i * ndim;
    double l3 = exp(v[0]), l4 = exp(v[1]), l5 = exp(v[2]), phi3 = v[3], phi4 = v[4], phi5 = v[5], m = v[6];
    double l3x = l3 * cos(phi3), l3y = l3 * sin(phi3);
    double l6 = l3 * l3 + l4 * l4 + l5 * l5 +
                2 * (l3 * l4 * cos(phi3 - phi4) - l3 * l5 * cos(phi3 - phi5) - l4 * l5 * cos(phi4 - phi5));
    l6 = l6 > 0 ? sqrt(l6) : 0;
    double res = 0;
    if (!(l6 <= 0 || l6 > c->lMax)) {
      double G = G_rect(c->p->thetaMax, side_y(c->p), l3x, l3y);
      res = uHat(l3 * th[2]) * uHat(l4 * th[3]) * uHat(l5 * th[4]) * uHat(l6 * th[5]);
      res *= trispectrum_los(c->t, m, l3, l4, l5, l6);
      res *= l3 * l4 * l5;
      res *= l3 * l4 * l5;
      res *= G;
    }
    fval[i] = res;
  }
  return 0;
}
int integrand_T7_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned, double* fval) {
  const HaloCtx* c = (const HaloCtx*)fdata;
  const double* th = c->th;
#pragma omp parallel for schedule(dynamic, 1) if (npts > 8)
  for (long i = 0; i < (long)npts; ++i) {
    const double* v = x + i * ndim;
    double l1 = exp(v[0]), l2 = exp(v[1]), l4 = exp(v[2]), l5 = exp(v[3]), phi1 = v[4], phi2 = v[5], m = v[6];
    double l3 = l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi1);
    double l6 = l4 * l4 + l5 * l5 + 2 * l4 * l5 * cos(phi2);
    double res = 0;
    if (!(l3 <= 0 || l6 <= 0)) {
      double l[6] = {l1, l2, sqrt(l3), l4, l5, sqrt(l6)};
      res = uHat(l[0] * th[0]) * uHat(l[1] * th[1]) * uHat(l[2] * th[2]) * uHat(l[3] * th[3]) * uHat(l[4] * th[4]) *
            uHat(l[5] * th[5]);
      res *= pentaspectrum_los(c->t, m, l);
      res *= l1 * l2 * l4 * l5;
      res *= l1 * l2 * l4 * l5;
    }
    fval[i] = res;
  }
  return 0;
}

// host lower bound of T5/T6/T7 (the reference sets its host lMin to 1e-4 there)
constexpr double HALO_LMIN = 1e-4;

}  // namespace

// the T5 / T6 / T7 integrand behind the cubature interface, for pinning the
// cubature on these integrands to the reference's own hcubature_v
struct orc_halo_ctx {
  HaloCtx c;
  orc_cov_params p;
  int term;
};
extern "C" orc_halo_ctx* orc_halo_ctx_create(const orc_tables* t, const orc_cov_params* p, int term, const double* th) {
  ensure_halo(t);
  orc_halo_ctx* h = new orc_halo_ctx();
  h->p = *p;
  h->term = term;
  double tmin123 = std::min({th[0], th[1], th[2]}), tmin456 = std::min({th[3], th[4], th[5]});
  double lMax = 10. / (term == 7 ? std::min(tmin123, tmin456) : std::max(tmin123, tmin456));
  h->c = HaloCtx{t, &h->p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  return h;
}
extern "C" void orc_halo_ctx_destroy(orc_halo_ctx* h) { delete h; }
extern "C" double orc_halo_ctx_lmax(const orc_halo_ctx* h) { return h->c.lMax; }
extern "C" int orc_integrand_halo_v(unsigned ndim, size_t npts, const double* x, void* fdata, unsigned fdim,
                                    double* fval) {
  orc_halo_ctx* h = (orc_halo_ctx*)fdata;
  if (h->term == 5) return integrand_T5_v(ndim, npts, x, &h->c, fdim, fval);
  if (h->term == 6) return integrand_T6_v(ndim, npts, x, &h->c, fdim, fval);
  return integrand_T7_v(ndim, npts, x, &h->c, fdim, fval);
}

extern "C" void orc_halo_tables(const orc_tables* t, double* out) {
  ensure_halo(t);
  std::memcpy(out, t->sig2, sizeof(double) * NM);
  std::memcpy(out + NM, t->dsig2, sizeof(double) * NM);
}
extern "C" double orc_hmf(const orc_tables* t, double m, double z) {
  ensure_halo(t);
  return hmf(t, m, z);
}
extern "C" void orc_sici(double x, double* si, double* ci) { sici(x, *si, *ci); }
extern "C" double orc_u_nfw(const orc_tables* t, double k, double m, double z) { return u_nfw(t, k, m, z); }
extern "C" double orc_concentration(double m, double z) { return concentration(m, z); }
extern "C" double orc_r_200(const orc_tables* t, double m) { return r_200(t, m); }
extern "C" double orc_get_sigma2(const orc_tables* t, double m, double z) {
  ensure_halo(t);
  return get_sigma2(t, m, z);
}
extern "C" double orc_get_dsigma2(const orc_tables* t, double m, double z) {
  ensure_halo(t);
  return get_dsigma2(t, m, z);
}
// line-of-sight tri-/pentaspectrum at points: pts rows (m, l1..l6); the
// trispectrum uses l1..l4
extern "C" void orc_halo_los(const orc_tables* t, const double* pts, long n, double* tri, double* penta) {
  ensure_halo(t);
#pragma omp parallel for schedule(dynamic, 1)
  for (long i = 0; i < n; ++i) {
    const double* r = pts + 7 * i;
    tri[i] = trispectrum_los(t, r[0], r[1], r[2], r[3], r[4]);
    penta[i] = pentaspectrum_los(t, r[0], r + 1);
  }
}
// integrand values of T5 (ndim 6), T6 (7) or T7 (7) at points x
extern "C" void orc_halo_integrand(const orc_tables* t, const orc_cov_params* p, int term, const double* th,
                                   double lMax, const double* x, long n, double* out) {
  ensure_halo(t);
  HaloCtx c{t, p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  if (term == 5) integrand_T5_v(6, (size_t)n, x, &c, 1, out);
  else if (term == 6) integrand_T6_v(7, (size_t)n, x, &c, 1, out);
  else integrand_T7_v(7, (size_t)n, x, &c, 1, out);
}

// T5 (:1199-1231, infinite survey), T6 (:1233-1276, square or rectangle: the
// 1-D T2 part-1 integral of (theta1, theta2) times a 7-D integral), T7
// (:1278-1313, infinite). relTol <= 0 selects the reference's tolerance (1e-2,
// 1e-1, 1e-1); maxEval 0 = unbounded, as the reference passes.
extern "C" double orc_T_halo(const orc_tables* t, const orc_cov_params* p, int term, const double* th, double relTol,
                             long maxEval, double* err_out, long* neval) {
  ensure_halo(t);
  double tmin123 = std::min({th[0], th[1], th[2]}), tmin456 = std::min({th[3], th[4], th[5]});
  double lMax = 10. / (term == 7 ? std::min(tmin123, tmin456) : std::max(tmin123, tmin456));
  HaloCtx c{t, p, {th[0], th[1], th[2], th[3], th[4], th[5]}, lMax};
  const double mmin = pow(10, LOGMMIN), mmax = pow(10, LOGMMAX);
  const double ll = log(HALO_LMIN), lh = log(lMax);
  double res = 0, err = 0;
  if (term == 5) {
    double xmin[6] = {ll, ll, ll, 0, 0, mmin}, xmax[6] = {lh, lh, lh, 2 * PI, 2 * PI, mmax};
    orc_hcubature_v(1, integrand_T5_v, &c, 6, xmin, xmax, (size_t)maxEval, 0, relTol > 0 ? relTol : 1e-2,
                    ORC_ERROR_L1, &res, &err);
    const double s = 1 / p->area / pow(2 * PI, 5);
    res *= s, err *= s;
  } else if (term == 6) {
    double xmin[7] = {ll, ll, ll, 0, 0, 0, mmin}, xmax[7] = {lh, lh, lh, 2 * PI, 2 * PI, 2 * PI, mmax};
    orc_hcubature_v(1, integrand_T6_v, &c, 7, xmin, xmax, (size_t)maxEval, 0, relTol > 0 ? relTol : 1e-1,
                    ORC_ERROR_L1, &res, &err);
    const long nev7 = orc_last_neval();
    // integral over ell_1: integrand_T2_part1 over [lMin, lMax] (:1247-1255)
    T2Ctx a{t, p, th[0], th[1], 1};
    orc_cov_params q = *p;
    q.lMin = 0;  // the device cut (dev_lMin) stays at the driver's 0
    a.p = &q;
    double vmin1[1] = {HALO_LMIN}, vmax1[1] = {lMax}, rA, eA;
    orc_hcubature_v(1, integrand_T2_v, &a, 1, vmin1, vmax1, 0, 0, 1e-4, ORC_ERROR_L1, &rA, &eA);
    rA /= 2 * PI;
    const double s = rA / pow(2 * PI, 6);
    res *= s, err *= fabs(s);
    if (neval) *neval = nev7;
    if (err_out) *err_out = err;
    return res;
  } else {
    double xmin[7] = {ll, ll, ll, ll, 0, 0, mmin}, xmax[7] = {lh, lh, lh, lh, 2 * PI, 2 * PI, mmax};
    orc_hcubature_v(1, integrand_T7_v, &c, 7, xmin, xmax, (size_t)maxEval, 0, relTol > 0 ? relTol : 1e-1,
                    ORC_ERROR_L1, &res, &err);
    const double s = 1 / p->area / pow(2 * PI, 6);
    res *= s, err *= s;
  }
  if (neval) *neval = orc_last_neval();
  if (err_out) *err_out = err;
  return res;
}

// T5_total (:685-845), T6_total (:847-1024), T7_total (:1026-1044) as sums
// of (multiplicity, argument pattern) over (a0, a1, a2, b0, b1, b2).
// T5_total tests a0 == a1 twice (:703-705), so with a0 == a1 the first
// triplet is taken as (a0, a0, a0) whatever a2 is; the reference's outputs
// are defined by that.
extern "C" int orc_halo_total_terms(int term, const double* A, const double* B, int* mult, int* idx) {
  struct P {
    int m, i[6];
  };
  std::vector<P> v;
  auto set = [&](std::initializer_list<P> l) {
    v.clear();
    for (const P& e : l) v.push_back(e);
  };
  const double a0 = A[0], a1 = A[1], a2 = A[2], b0 = B[0], b1 = B[1], b2 = B[2];
  if (term == 7) {
    set({{1, {0, 1, 2, 3, 4, 5}}});
  } else if (term == 5) {
    if (a0 == a1) {
      if (b0 == b1 && b0 == b2) set({{9, {0, 0, 0, 3, 3, 3}}});
      else if (b0 == b1) set({{6, {0, 0, 0, 3, 3, 5}}, {3, {0, 0, 0, 5, 3, 3}}});
      else if (b1 == b2) set({{3, {0, 0, 0, 3, 4, 4}}, {6, {0, 0, 0, 4, 3, 4}}});
      else set({{3, {0, 0, 0, 3, 4, 5}}, {3, {0, 0, 0, 4, 3, 5}}, {3, {0, 0, 0, 5, 3, 4}}});
    } else if (b0 == b1 && b0 == b2) {
      set({{3, {0, 1, 2, 3, 3, 3}}, {3, {1, 0, 2, 3, 3, 3}}, {3, {2, 0, 1, 3, 3, 3}}});
    } else if (b0 == b1) {
      set({{2, {0, 1, 2, 3, 3, 5}}, {1, {0, 1, 2, 5, 3, 3}}, {2, {1, 0, 2, 3, 4, 5}},
           {1, {1, 0, 2, 5, 3, 3}}, {2, {2, 0, 1, 3, 3, 5}}, {1, {2, 0, 1, 5, 3, 3}}});
    } else if (b1 == b2) {
      set({{1, {0, 1, 2, 3, 4, 4}}, {2, {0, 1, 2, 4, 3, 4}}, {1, {1, 0, 2, 3, 4, 4}},
           {2, {1, 0, 2, 4, 3, 4}}, {1, {2, 0, 1, 3, 4, 4}}, {2, {2, 0, 1, 4, 3, 4}}});
    } else {
      for (auto f : {std::array<int, 3>{0, 1, 2}, {1, 0, 2}, {2, 0, 1}})
        for (auto s : {std::array<int, 3>{3, 4, 5}, {4, 3, 5}, {5, 3, 4}}) v.push_back({1, {f[0], f[1], f[2], s[0], s[1], s[2]}});
    }
  } else if (term == 6) {
    if (a0 == a1 && a0 == a2) {
      if (b0 == b1 && b0 == b2) set({{3, {0, 0, 0, 3, 3, 3}}, {3, {3, 3, 0, 0, 0, 3}}});
      else if (b0 == b1) set({{3, {0, 0, 0, 3, 3, 5}}, {1, {3, 3, 0, 0, 0, 5}}, {2, {3, 5, 0, 0, 0, 3}}});
      else if (b1 == b2) set({{3, {0, 0, 0, 3, 4, 4}}, {2, {3, 4, 0, 0, 0, 4}}, {1, {4, 4, 0, 0, 0, 3}}});
      else set({{3, {0, 0, 0, 3, 4, 5}}, {1, {3, 4, 0, 0, 0, 5}}, {1, {3, 5, 0, 0, 0, 4}}, {1, {4, 5, 0, 0, 0, 3}}});
    } else if (a0 == a1) {
      if (b0 == b1 && b0 == b2) set({{1, {0, 0, 2, 3, 3, 3}}, {2, {0, 2, 0, 3, 3, 3}}, {3, {3, 3, 0, 0, 2, 3}}});
      else if (b0 == b1)
        set({{1, {0, 0, 2, 3, 3, 5}}, {2, {0, 2, 0, 3, 3, 5}}, {1, {3, 3, 0, 0, 2, 5}}, {2, {3, 5, 0, 0, 2, 3}}});
      else if (b1 == b2)
        set({{1, {0, 0, 2, 3, 4, 4}}, {2, {0, 2, 0, 3, 4, 4}}, {2, {3, 4, 0, 0, 2, 4}}, {1, {4, 4, 0, 0, 2, 3}}});
      else
        set({{1, {0, 0, 2, 3, 4, 5}}, {2, {0, 2, 0, 3, 4, 5}}, {1, {3, 4, 0, 0, 2, 5}},
             {1, {3, 5, 0, 0, 2, 4}}, {1, {4, 5, 0, 0, 2, 3}}});
    } else if (b0 == b1 && b0 == b2) {
      set({{1, {0, 1, 2, 3, 3, 3}}, {1, {0, 2, 1, 3, 3, 3}}, {1, {1, 2, 0, 3, 3, 3}}, {3, {3, 3, 0, 1, 2, 3}}});
    } else if (b0 == b1) {
      set({{1, {0, 1, 2, 3, 3, 5}}, {1, {0, 2, 1, 3, 3, 5}}, {1, {1, 2, 0, 3, 3, 5}},
           {1, {3, 3, 0, 1, 2, 5}}, {2, {3, 5, 0, 1, 2, 3}}});
    } else if (b1 == b2) {
      set({{1, {0, 1, 2, 3, 4, 4}}, {1, {0, 2, 1, 3, 4, 4}}, {1, {1, 2, 0, 3, 4, 4}},
           {2, {3, 4, 0, 1, 2, 4}}, {1, {4, 4, 0, 1, 2, 3}}});
    } else {
      set({{1, {0, 1, 2, 3, 4, 5}}, {1, {0, 2, 1, 3, 4, 5}}, {1, {1, 2, 0, 3, 4, 5}},
           {1, {3, 4, 0, 1, 2, 5}}, {1, {3, 5, 0, 1, 2, 4}}, {1, {4, 5, 0, 1, 2, 3}}});
    }
  } else {
    return -1;
  }
  for (size_t k = 0; k < v.size(); ++k) {
    mult[k] = v[k].m;
    for (int j = 0; j < 6; ++j) idx[6 * k + j] = v[k].i[j];
  }
  return (int)v.size();
}

// T5/T6/T7 totals with each distinct argument set integrated once
extern "C" double orc_T_halo_total(const orc_tables* t, const orc_cov_params* p, int term, const double* A,
                                   const double* B, double relTol, long maxEval) {
  if (term == 6 && p->type == 2) return 0;  // T6_total, :849-850
  int mult[16], idx[96];
  int n = orc_halo_total_terms(term, A, B, mult, idx);
  const double src[6] = {A[0], A[1], A[2], B[0], B[1], B[2]};
  double r = 0;
  for (int k = 0; k < n; ++k) {
    double th[6];
    for (int j = 0; j < 6; ++j) th[j] = src[idx[6 * k + j]];
    r += mult[k] * orc_T_halo(t, p, term, th, relTol, maxEval, nullptr, nullptr);
  }
  return r;
}
