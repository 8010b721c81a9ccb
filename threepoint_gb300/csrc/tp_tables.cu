// GPU builder of the per-cosmology FP64 tables (the reference's host-side
// set_cosmology, cuda_version/bispectrum.cu:100-219) and of the per-node
// line-of-sight coefficients used by the integrand kernels.
//
// Layout in HBM: one TablesDev (~14 KB) per cosmology; one NC_COUNT x 96
// double block (+ a float copy) of b_kappa node coefficients and one
// HC_COUNT x 96 double block of Halofit node coefficients per cosmology.
#include <math.h>

#include "tp_bispec.cuh"
#include "tp_internal.cuh"
#include "tp_kernels.cuh"
#include "tp_tables.cuh"

namespace tp {

__constant__ double c_gq_a[48];  // Gauss-Legendre abscissae on (0,1), ascending
__constant__ double c_gq_w[48];

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
void gauss_legendre96(double* a48, double* w48) {
  const int n = 96;
  for (int i = 0; i < 48; ++i) {
    long double x = cosl(3.14159265358979323846264338327950288L * (48 - i - 0.25L) / (n + 0.5L));
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
    long double p0 = 1, p1 = x;
    for (int k = 2; k <= n; ++k) {
      long double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (x * p1 - p0) / (x * x - 1);
    a48[i] = (double)x;
    w48[i] = (double)(2.0L / ((1 - x * x) * dp * dp));
  }
}

// cosmology-only part of the Eisenstein & Hu fit (bispectrum.cu:651-686)
EHConst make_eh_const(const CosmoDev& c, double norm) {
  EHConst e;
  double fc = c.omc / c.om, fb = c.omb / c.om;
  double theta = 2.728 / 2.7;
  double pc = 0.25 * (5.0 - sqrt(1.0 + 24.0 * fc));
  double omh2 = c.om * c.h * c.h, ombh2 = c.omb * c.h * c.h;
  double zeq = 2.5e+4 * omh2 / pow(theta, 4);
  double b1 = 0.313 * pow(omh2, -0.419) * (1.0 + 0.607 * pow(omh2, 0.674));
  double b2 = 0.238 * pow(omh2, 0.223);
  double zd = 1291.0 * pow(omh2, 0.251) / (1.0 + 0.659 * pow(omh2, 0.828)) * (1.0 + b1 * pow(ombh2, b2));
  double yd = (1.0 + zeq) / (1.0 + zd);
  double sh = 44.5 * log(9.83 / omh2) / sqrt(1.0 + 10.0 * pow(ombh2, 0.75));
  double alnu = fc * (5.0 - 2.0 * pc) / 5.0 * (1.0 - 0.553 * fb + 0.126 * fb * fb * fb) * pow(1.0 + yd, -pc) *
                (1.0 + 0.5 * pc * (1.0 + 1.0 / (7.0 * (3.0 - 4.0 * pc))) / (1.0 + yd));
  e.h = c.h;
  e.omh2 = omh2;
  e.theta2 = theta * theta;
  e.sa = sqrt(alnu);
  e.one_m_sa = 1.0 - e.sa;
  e.sh = sh;
  e.c184 = 1.84 * e.sa / (1.0 - 0.949 * fb);
  // P(k) [h^-3 Mpc^3] = h^3 2 pi^2 norm^2 (2997.9/h)^(3+ns) * kk^ns * (L/(L+C q^2))^2
  e.ehc = c.h * c.h * c.h * 2.0 * PI * PI * norm * norm * pow(2997.9 / c.h, 3. + c.ns);
  e.ns = c.ns;
  return e;
}

// ---------------------------------------------------------------------------
// device FP64 physics of the table build
// ---------------------------------------------------------------------------
__device__ inline double d_E(const CosmoDev& c, double z) {
  return sqrt(c.om * pow(1 + z, 3.0) + c.ow * pow(1 + z, 3 * (1.0 + c.w)));
}

// linear_pk, bispectrum.cu:602-693 (table branch or hoisted Eisenstein & Hu)
__device__ inline double d_linear_pk(const CosmoDev& c, const EHConst& e, const double* pk, double k) {
  if (c.pk_given) {
    if (k >= c.kmax) return pk[NK - 1];
    if (k <= c.kmin) return pk[0];
    double didx = log(k / c.kmin) / c.dk;
    int idx = (int)didx;
    didx -= idx;
    if (idx >= NK - 1) return pk[NK - 1];
    return pk[idx] * (1 - didx) + pk[idx + 1] * didx;
  }
  return eh_linear_pk(e, k);
}

// window functions, bispectrum.cu:854-868
__device__ inline double d_window(double x, int i) {
  if (i == 0) return 3.0 / (x * x * x) * (sin(x) - x * cos(x));
  if (i == 1) return exp(-0.5 * x * x);
  if (i == 2) return x * exp(-0.5 * x * x);
  if (i == 3) return x * x * (1 - x * x) * exp(-x * x);
  return (3 * (x * x - 3) * sin(x) + 9 * x * cos(x)) / x / x / x / x;
}

// Eisenstein & Hu no-wiggle transfer function L / (L + C q^2) at k [h/Mpc]
// (bispectrum.cu:602-693, the k-dependent factor of linear_pk)
__device__ __noinline__ double eh_transfer(const EHConst& e, double k) {
  const double kk = k * e.h;
  const double xs = 0.43 * kk * e.sh;
  const double xs2 = xs * xs;
  const double geff = e.omh2 * (e.sa + e.one_m_sa / (1.0 + xs2 * xs2));
  const double qeff = kk / geff * e.theta2;
  const double L = log(2.718281828 + e.c184 * qeff);
  const double C = 14.4 + 325.0 / (1.0 + 60.5 * exp(1.11 * log(qeff)));
  return L / (L + C * qeff * qeff);
}

// 2 ln T(e^t) from one cosmology's EHG table by 4-point Lagrange
// interpolation; false outside the grid's interior (or for a NaN t)
__device__ inline bool eh_table_lookup(const double* __restrict__ g, double t, double& out) {
  const double x = (t - EHG_T0) * EHG_PER_UNIT;
  if (!(x >= 1.0 && x < (double)(EHG_N - 2))) return false;
  const int i = (int)x;
  const double u = x - i, um1 = u - 1.0, um2 = u - 2.0, up1 = u + 1.0;
  const double a = u * um1, b = up1 * um2;
  // weights -a(u-2)/6, b(u-1)/2, -b u/2, a(u+1)/6 on g[i-1], g[i], g[i+1], g[i+2]
  out = a * (up1 * g[i + 2] - um2 * g[i - 1]) * (1.0 / 6.0) + b * (um1 * g[i] - u * g[i + 1]) * 0.5;
  return true;
}

// Integrand in ln k of sigmam (bispectrum.cu:823-832): k^3 P(k) W(kr)^2 for
// j < 3, k^3 P(k) W(kr) for j = 3, at k = exp(t). For the Gaussian windows
// (j = 1..3) the powers k^3, (kh)^ns, exp(-(kr)^2) and the squared transfer
// function are folded into one exp; the values agree with the literal form
// to rounding. ehg (or null) is the cosmology's EHG table of 2 ln T, used
// inside its grid: the integrand then agrees with the formula to 3e-13.
__device__ inline double sigma_integrand(const CosmoDev& c, const EHConst& e, const double* pk, double k, double t,
                                         double r, int j, double lnh, double lnkmin, const double* ehg) {
  if (j == 0) {
    double w = d_window(k * r, 0);
    return k * k * k * d_linear_pk(c, e, pk, k) * w * w;
  }
  const double x2 = (k * r) * (k * r);
  double v;
  if (c.pk_given) {
    double p;
    if (k >= c.kmax) {
      p = pk[NK - 1];
    } else if (k <= c.kmin) {
      p = pk[0];
    } else {
      double didx = (t - lnkmin) / c.dk;
      int idx = (int)didx;
      didx -= idx;
      p = idx >= NK - 1 ? pk[NK - 1] : pk[idx] * (1 - didx) + pk[idx + 1] * didx;
    }
    v = exp(3.0 * t - x2) * p;
  } else {
    // Eisenstein & Hu no-wiggle shape (bispectrum.cu:602-693) times k^3 W^2
    double g2;
    if (ehg && eh_table_lookup(ehg, t, g2)) {
      v = e.ehc * exp((3.0 + e.ns) * t + e.ns * lnh - x2 + g2);
    } else {
      const double rr = eh_transfer(e, k);
      v = e.ehc * exp((3.0 + e.ns) * t + e.ns * lnh - x2) * rr * rr;
    }
  }
  if (j == 1) return v;
  if (j == 2) return v * x2;
  return v * x2 * (1 - x2);
}

// sigma(R): nested doubling trapezoid in ln k (bispectrum.cu:796-852). All 32
// lanes of the calling warp cooperate on the trapezoid sums and return the
// same value (xor-butterfly sums are bitwise identical in every lane). Each
// doubling evaluates only the new odd points and adds them to the previous
// level's sum: the even points of level n are bitwise the points of level n/2
// (hh is halved exactly), so this is the reference's sum in another order.
__device__ double warp_sigmam(const CosmoDev& c, const EHConst& e, const double* pk, double r, int j,
                              const double* ehg = nullptr) {
  if (c.sigma8 < 1e-8) return 0;
  const int lane = threadIdx.x & 31;
  const double lnh = log(e.h), lnkmin = c.pk_given ? log(c.kmin) : 0.0;
  double k1 = 2. * PI / r, k2 = 2. * PI / r;
  double xx = 0, xxpp = -1.0;
  const bool run_k = ehg && j > 0 && !c.pk_given;
  // iteration caps: at most 2^22 trapezoid points per pass; a non-finite sum
  // (only for invalid cosmologies) ends the iteration
  for (int outer = 0; outer < 40; ++outer) {
    k1 = k1 / 10.0;
    k2 = k2 * 2.0;
    double a = log(k1), b = log(k2);
    double xxp = -1.0;
    int n = 2;
    double ends = 0.5 * (sigma_integrand(c, e, pk, k1, a, r, j, lnh, lnkmin, ehg) +
                         sigma_integrand(c, e, pk, k2, b, r, j, lnh, lnkmin, ehg));
    double sum = 0;
    for (int inner = 0; inner < 21; ++inner) {
      n = n * 2;
      double hh = (b - a) / (double)n;
      double part = 0;
      if (n == 4) {  // first level: all three interior points
        for (int i = 1 + lane; i < 4; i += 32) {
          double t = a + hh * i;
          part += sigma_integrand(c, e, pk, exp(t), t, r, j, lnh, lnkmin, ehg);
        }
      } else if (run_k) {
        // k = e^t by a running product along the lane's points (a relative
        // error below 1e-14 in k, which enters only through exp(-(kr)^2))
        if (lane < n / 2) {
          const double step = exp(64.0 * hh);
          double k = exp(a + hh * (2 * lane + 1));
          for (int m = lane; m < n / 2; m += 32) {
            const double t = a + hh * (2 * m + 1);
            part += sigma_integrand(c, e, pk, k, t, r, j, lnh, lnkmin, ehg);
            k *= step;
          }
        }
      } else {
        for (int m = lane; m < n / 2; m += 32) {
          double t = a + hh * (2 * m + 1);
          part += sigma_integrand(c, e, pk, exp(t), t, r, j, lnh, lnkmin, ehg);
        }
      }
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      sum += part;
      xx = (sum + ends) * hh;
      if (!isfinite(xx) || fabs((xx - xxp) / xx) < EPS) break;
      xxp = xx;
    }
    if (!isfinite(xx) || fabs((xx - xxpp) / xx) < EPS) break;
    xxpp = xx;
  }
  if (j < 3) return sqrt(xx / (2.0 * PI * PI));
  return xx / (2.0 * PI * PI);
}

// growth ODE, bispectrum.cu:726-794
__device__ inline double d_lgr_rhs(const CosmoDev& c, double la, double y0, double y1) {
  double a = exp(la);
  double ap = pow(a, -3. * c.w);
  double g = -0.5 * (5. * c.om + (5. - 3 * c.w) * c.ow * ap) * y1 - 1.5 * (1. - c.w) * c.ow * ap * y0;
  return g / (c.om + c.ow * ap);
}
__device__ double d_lgr(const CosmoDev& c, double z) {
  double a = 1. / (1. + z), a0 = 1. / 1100.;
  double yp = -1., y0 = 1, y1 = 0;
  int n = 10;
  for (int it = 0; it < 20; ++it) {  // at most 10*2^20 RK4 steps
    n *= 2;
    double h = (log(a) - log(a0)) / n;
    double x = log(a0);
    y0 = 1.;
    y1 = 0.;
    for (int i = 0; i < n; i++) {
      double k10 = h * y1, k11 = h * d_lgr_rhs(c, x, y0, y1);
      double a0_ = y0 + 0.5 * k10, a1_ = y1 + 0.5 * k11;
      double k20 = h * a1_, k21 = h * d_lgr_rhs(c, x + 0.5 * h, a0_, a1_);
      double b0_ = y0 + 0.5 * k20, b1_ = y1 + 0.5 * k21;
      double k30 = h * b1_, k31 = h * d_lgr_rhs(c, x + 0.5 * h, b0_, b1_);
      double c0_ = y0 + k30, c1_ = y1 + k31;
      double k40 = h * c1_, k41 = h * d_lgr_rhs(c, x + h, c0_, c1_);
      y0 += (k10 + k40) / 6. + (k20 + k30) / 3.;
      y1 += (k11 + k41) / 6. + (k21 + k31) / 3.;
      x += h;
    }
    if (!isfinite(y0) || fabs(y0 / yp - 1.) < 0.1 * EPS) break;
    yp = y0;
  }
  return a * y0;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// The table kernels run as one-warp blocks of at most TP_TABLES_MAXNREG
// registers a thread. An SM's registers are split between its four
// sub-partitions (16384 each) and a warp takes its registers from one of
// them: three resident k_map3<float> CTAs (6 warps of 80 registers per
// sub-partition) leave 1024 registers in each, room for one 32-register
// warp. With the cap the next batch's tables build on the FP64 pipe while
// the current batch integrates, at the cost of spills to L1.
#ifndef TP_TABLES_MAXNREG
#define TP_TABLES_MAXNREG 32
#endif
#define TP_TABLE_KERNEL __global__ void __maxnreg__(TP_TABLES_MAXNREG)

// The table build reads the Eisenstein & Hu P(k) even when a linear P(k)
// table is given, as the reference does: its set_cosmology declares a local
// Pk_given (cuda_version/bispectrum.cu:132) that shadows the global flag its
// host linear_pk reads (:36, :623), so norm, r_sigma, n_eff and ncur come from
// Eisenstein & Hu and only the bispectrum's linear P(k) reads the table
// (dev_Pk_given, :605-621). tables_cosmo() is the cosmology the build sees.
__device__ __forceinline__ CosmoDev tables_cosmo(const CosmoDev& in) {
  CosmoDev c = in;
  c.pk_given = 0;
  return c;
}

// norm = sigma8 / sigma(8 Mpc/h, top hat) and the growth integral at z = 0;
// one warp per cosmology
TP_TABLE_KERNEL k_norm(const CosmoDev* cos, EHConst* eh, TablesDev* tab, int n) {
  int ci = blockIdx.x;
  if (ci >= n) return;
  const CosmoDev c = tables_cosmo(cos[ci]);
  EHConst e = eh[ci];  // built with norm = 1
  double s = warp_sigmam(c, e, tab[ci].pk, 8., 0);
  if (threadIdx.x == 0) {
    double norm = c.sigma8 / s;
    tab[ci].norm = norm;
    tab[ci].dz = c.zmax / NZ;
    eh[ci].ehc = e.ehc * norm * norm;
    tab[ci].lgr0 = d_lgr(c, 0.);
  }
}

// f_K on bin centres (bispectrum.cu:158-166); block b of a cosmology takes
// bins 32 b .. 32 b + 31
TP_TABLE_KERNEL k_fk(const CosmoDev* cos, TablesDev* tab, int n) {
  const int ci = blockIdx.x / (NZ / 32), i = (blockIdx.x % (NZ / 32)) * 32 + threadIdx.x;
  if (ci >= n) return;
  const CosmoDev c = cos[ci];
  const double dz = c.zmax / NZ;
  double zb = (i + 0.5) * dz;
  double cx = zb / 2, dx = zb / 2, q = 0;
  for (int m = 0; m < 48; m++) q += c_gq_w[m] * (1. / d_E(c, cx - dx * c_gq_a[m]) + 1. / d_E(c, cx + dx * c_gq_a[m]));
  tab[ci].f_K[i] = C_OVER_H0 * (q * dx);
}

// lensing efficiency g by the trapezoid sum over n(z) (bispectrum.cu:168-190)
TP_TABLE_KERNEL k_g(const CosmoDev* cos, const double* nz, int nz_stride, TablesDev* tab, int n) {
  const int ci = blockIdx.x / (NZ / 32), i = (blockIdx.x % (NZ / 32)) * 32 + threadIdx.x;
  if (ci >= n) return;
  const double dz = cos[ci].zmax / NZ;
  TablesDev& t = tab[ci];
  const double* fk = t.f_K;
  const double* nzc = nz + (size_t)ci * nz_stride;
  double gi = 0;
  for (int j = i; j < NZ; j++) {
    double term = nzc[j] * (fk[j] - fk[i]) / fk[j];
    gi += (j == i || j == NZ - 1) ? term / 2 : term;
  }
  t.g[i] = (i == 0) ? 1.0 : gi * dz;
}

// linear growth D1 = lgr(z)/lgr(0) on bin centres (bispectrum.cu:207)
TP_TABLE_KERNEL k_growth(const CosmoDev* cos, TablesDev* tab, int n) {
  const int ci = blockIdx.x / (NZ / 32), i = (blockIdx.x % (NZ / 32)) * 32 + threadIdx.x;
  if (ci >= n) return;
  const CosmoDev c = cos[ci];
  tab[ci].D1[i] = d_lgr(c, (i + 0.5) * (c.zmax / NZ)) / tab[ci].lgr0;
}

// 2 ln T(k) of the Eisenstein & Hu fit on the EHG grid, one thread per
// (cosmology, grid point); shape constants only, so it runs before k_norm
TP_TABLE_KERNEL k_eh_table(const CosmoDev* cos, const EHConst* eh, double* ehg, int n) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ci = (int)(idx / EHG_N), i = (int)(idx % EHG_N);
  if (ci >= n) return;
  const double t = EHG_T0 + i / EHG_PER_UNIT;
  ehg[(size_t)ci * EHG_N + i] = 2.0 * log(eh_transfer(eh[ci], exp(t)));
}

// r_sigma by bisection on D1 sigma(1/k) = 1, then n_eff and ncur
// (bispectrum.cu:202-212, 870-903). One warp takes RS_BINS adjacent redshift
// bins of a cosmology; lane b < RS_BINS holds bin b's bisection as a state
// machine that advances one iteration of the one-bin loops per round. sigma(R)
// does not depend on the bin, and while adjacent bins' brackets coincide they
// ask for sigma at bitwise the same k: each round the warp evaluates every
// distinct k once (all 32 lanes in the trapezoid sums) and hands the value to
// the bins that asked for it. Every bin sees the same sequence of values and
// makes the same decisions as alone, with ~40% fewer sigma(R) integrals.
constexpr int RS_BINS = 8;
static_assert(NZ % RS_BINS == 0 && RS_BINS <= 32, "bins per warp");

TP_TABLE_KERNEL k_rsigma(const CosmoDev* cos, const EHConst* eh, TablesDev* tab, const double* ehg_all, int n) {
  const unsigned FULL = 0xffffffffu;
  const int ci = blockIdx.x / (NZ / RS_BINS), b0 = (blockIdx.x % (NZ / RS_BINS)) * RS_BINS;
  if (ci >= n) return;
  const int lane = threadIdx.x & 31;
  const CosmoDev c = tables_cosmo(cos[ci]);
  const EHConst e = eh[ci];
  TablesDev& t = tab[ci];
  const double* pk = t.pk;
  const double* ehg = ehg_all + (size_t)ci * EHG_N;
  const bool mine = lane < RS_BINS;
  const int bin = b0 + (mine ? lane : 0);
  const double D1 = t.D1[bin];
  // phase 0: k1 halving (<= 100 steps), 1: k2 doubling (<= 100), 2: bisection
  // (<= 200), 3: done; the loop limits and exits of the one-bin version
  enum { HALVE = 0, DOUBLE = 1, BISECT = 2, DONE = 3 };
  double k1 = 1., k2 = 1., k = 0.;
  int phase = DONE, it = 0;
  bool bad = false;
  if (mine && c.sigma8 >= 1e-8) {
    bad = !isfinite(D1);
    phase = bad ? DONE : HALVE;
  }
  for (int round = 0; round < 400; ++round) {
    const double kq = phase == HALVE ? k1 : phase == DOUBLE ? k2 : 0.5 * (k1 + k2);
    unsigned pending = __ballot_sync(FULL, phase != DONE);
    if (!pending) break;
    double sg = 0;
    while (pending) {
      const double kv = __shfl_sync(FULL, kq, __ffs(pending) - 1);
      const double v = warp_sigmam(c, e, pk, 1. / kv, 1, ehg);
      const bool match = ((pending >> lane) & 1u) && kq == kv;
      if (match) sg = v;
      pending &= ~__ballot_sync(FULL, match);
    }
    if (phase == DONE) continue;
    const double s = D1 * sg;
    if (phase == HALVE) {
      if (!isfinite(s)) bad = true;
      if (s < 1. || bad) {
        phase = bad ? DONE : DOUBLE;
        it = 0;
      } else {
        k1 *= 0.5;
        if (++it == 100) phase = DOUBLE, it = 0;
      }
    } else if (phase == DOUBLE) {
      if (!isfinite(s)) bad = true;
      if (s > 1. || bad) {
        phase = bad ? DONE : BISECT;
        it = 0;
      } else {
        k2 *= 2.;
        if (++it == 100) phase = BISECT, it = 0;
      }
    } else {
      k = kq;
      if (!isfinite(s)) {
        bad = true;
        phase = DONE;
      } else {
        if (s < 1.)
          k1 = k;
        else if (s > 1.)
          k2 = k;
        if (s == 1. || fabs(k2 / k1 - 1.) < EPS * 0.1 || ++it == 200) phase = DONE;
      }
    }
  }
  const double rs = (c.sigma8 >= 1e-8) ? (bad ? NAN : 1. / k) : 0.0;
  // n_eff and ncur need sigma at each bin's own radius: one bin after another
  double s2 = NAN, s3 = NAN;
  for (int b = 0; b < RS_BINS; ++b) {
    const double rb = __shfl_sync(FULL, rs, b);
    if (!isfinite(rb)) continue;
    const double v2 = warp_sigmam(c, e, pk, rb, 2, ehg);
    const double v3 = warp_sigmam(c, e, pk, rb, 3, ehg);
    if (lane == b) s2 = v2, s3 = v3;
  }
  if (mine) {
    double d1 = -2. * (D1 * s2) * (D1 * s2);
    t.r_sigma[bin] = rs;
    t.n_eff[bin] = -3. + 2. * (D1 * s2) * (D1 * s2);
    t.ncur[bin] = d1 * d1 + 4. * s3 * D1 * D1;
  }
}

// mid-bin two-point interpolation of a z table (bispectrum.cu:335-437) with
// the lower neighbour clamped at bin 0
__device__ inline double interp_mid(const double* arr, double zfrac_bins) {
  int idx = (int)zfrac_bins;
  double didx = zfrac_bins - idx;
  if (idx > NZ - 1) {
    idx = NZ - 1;
    didx = 1.0;
  }
  int ii = idx;
  double w = 1 - fabs(didx - 0.5), iw = 1 - w;
  if (didx > 0.5) {
    if (idx == NZ - 1)
      iw = 0.0;
    else
      ii = idx + 1;
  } else if (didx < 0.5) {
    ii = idx - 1 < 0 ? 0 : idx - 1;
  }
  return arr[idx] * w + arr[ii] * iw;
}

// Per-node coefficients of b_kappa's LOS integral (z-only parts of
// integrand_bkappa + bispec, bispectrum.cu:221-333) and of P_kappa's
// (limber_integrand_power_spectrum + P_k_nonlinear, bispectrum.cu:531-600,951-991).
TP_TABLE_KERNEL k_node_coefs(const CosmoDev* cos, const TablesDev* tab, double* ncoef, float* ncoef_f, float* fcoef_f,
                             double* hcoef, float* hcoef_f, int n) {
  // one warp per 32 nodes of a cosmology
  int ci = blockIdx.x / (NNODE / 32);
  int j = (blockIdx.x % (NNODE / 32)) * 32 + threadIdx.x;
  if (ci >= n || j >= NNODE) return;
  const CosmoDev c = cos[ci];
  const TablesDev& t = tab[ci];
  int i = j >> 1;
  double cx = c.zmax / 2, dx = c.zmax / 2;
  double z = (j & 1) ? cx + dx * c_gq_a[i] : cx - dx * c_gq_a[i];
  double wq = c_gq_w[i] * dx;

  // ---- b_kappa nodes: interpolation index z/zmax*256 (bispectrum.cu:320)
  {
    double fb = z / c.zmax * NZ;
    double g = interp_mid(t.g, fb), fK = interp_mid(t.f_K, fb);
    double D1 = interp_mid(t.D1, fb), rs = interp_mid(t.r_sigma, fb), ne = interp_mid(t.n_eff, fb);
    double E = d_E(c, z);
    double pref = 27. / 8. * c.om * c.om * c.om * pow(H0_OVER_C, 5.0);
    double gz = g * (1. + z);
    double W = (z < 1.0e-7) ? 0.0 : wq * pref * gz * gz * gz / fK / E;
    double ls = log10(D1 * c.sigma8);
    double a = 1. / (1. + z);
    double omz = c.om / (c.om + c.ow * pow(a, -3. * c.w));
    double v[NC_COUNT];
    v[NC_W] = W;
    v[NC_S] = rs / fK;
    v[NC_L2S] = log2(rs / fK);
    v[NC_HF] = c.h / fK;
    v[NC_L2HF] = log2(c.h / fK);
    v[NC_ANA] = LOG2_10 * (-2.167 - 2.944 * ls - 1.106 * ls * ls - 2.865 * ls * ls * ls);
    v[NC_ANR] = 0.310 * LOG2_10;
    v[NC_ANC] = pow(10., 0.182 + 0.57 * ne);
    v[NC_BN] = pow(10., -3.428 - 2.681 * ls + 1.624 * ls * ls - 0.095 * ls * ls * ls);
    v[NC_CN] = pow(10., 0.159 - 1.107 * ne);
    v[NC_ALA] = LOG2_10 * (-4.348 - 3.006 * ne - 0.5745 * ne * ne);
    v[NC_ALD] = LOG2_10 * pow(10., -0.9 + 0.2 * ne);
    v[NC_BETAB] = pow(10., -1.731 - 2.845 * ne - 1.4995 * ne * ne - 0.2811 * ne * ne * ne);
    v[NC_FN] = pow(10., -10.533 - 16.838 * ne - 9.3048 * ne * ne - 1.8263 * ne * ne * ne);
    v[NC_GN] = pow(10., 2.787 + 2.405 * ne + 0.4577 * ne * ne);
    v[NC_HN] = pow(10., -1.118 - 0.394 * ne);
    v[NC_MN] = pow(10., -2.605 - 2.434 * ls + 5.71 * ls * ls);
    v[NC_NN] = pow(10., -4.468 - 3.08 * ls + 1.035 * ls * ls);
    v[NC_MUN] = pow(10., 15.312 + 22.977 * ne + 10.9579 * ne * ne + 1.6586 * ne * ne * ne);
    v[NC_NUN] = pow(10., 1.347 + 1.246 * ne + 0.4525 * ne * ne);
    v[NC_PN] = pow(10., 0.071 - 0.433 * ne);
    v[NC_EN] = pow(10., -0.632 + 0.646 * ne);
    v[NC_DN] = pow(10., -0.483 + 0.892 * ls - 0.086 * omz);
    v[NC_D1SQ] = D1 * D1;
    v[NC_TREE] = z > 10. ? 1.0 : 0.0;
    v[NC_D1P4] = D1 * D1 * D1 * D1;
    double* o = ncoef + ((size_t)ci * NNODE + j) * NCP;
    float* of = ncoef_f + ((size_t)ci * NNODE + j) * NCP;
    for (int q = 0; q < NCP; ++q) {
      o[q] = q < NC_COUNT ? v[q] : 0.0;
      of[q] = q < NC_COUNT ? (float)v[q] : 0.f;
    }
    // folded FP32 row of the point path (NF_*); NF_W is normalised in k_finish
    const double sq = rs / fK, hf = c.h / fK;
    double f[NF_COUNT];
    f[NF_W] = W;
    f[NF_L2S] = log2(sq);
    f[NF_L2HF] = log2(hf);
    f[NF_HF] = hf;
    f[NF_TOFF] = (log2(hf) - PLT_LO) * ((PLT_N - 1) / (PLT_HI - PLT_LO));
    f[NF_ANA] = v[NC_ANA];
    f[NF_L2ANR] = log2(v[NC_ANR]);
    f[NF_ANC] = v[NC_ANC];
    f[NF_L2BN] = LOG2_10 * (-3.428 - 2.681 * ls + 1.624 * ls * ls - 0.095 * ls * ls * ls);
    f[NF_CNS] = v[NC_CN] * sq;
    f[NF_ALA] = v[NC_ALA];
    f[NF_ALD] = v[NC_ALD];
    f[NF_BETAB] = v[NC_BETAB];
    f[NF_D1SQ] = D1 * D1;
    f[NF_D1SQFNS2] = D1 * D1 * v[NC_FN] * sq * sq;
    f[NF_GNS] = v[NC_GN] * sq;
    f[NF_HNS2] = v[NC_HN] * sq * sq;
    f[NF_L2MN] = LOG2_10 * (-2.605 - 2.434 * ls + 5.71 * ls * ls);
    f[NF_L2NN] = LOG2_10 * (-4.468 - 3.08 * ls + 1.035 * ls * ls);
    f[NF_MUN] = v[NC_MUN];
    f[NF_NUN] = v[NC_NUN];
    f[NF_PNS] = v[NC_PN] * sq;
    f[NF_ENS] = v[NC_EN] * sq;
    f[NF_DNS] = v[NC_DN] * sq;
    f[NF_TREE] = v[NC_TREE];
    f[NF_D1P4] = v[NC_D1P4];
    // pair-interleaved layout (nf_index): nodes 2p and 2p+1 side by side
    float* ff = fcoef_f + (size_t)ci * NNODE * NCP;
    for (int q = 0; q < NCP; ++q) ff[nf_index(j, q)] = q < NF_COUNT ? (float)f[q] : 0.f;
  }
  // ---- P_kappa nodes: interpolation index z/zmax*255 (bispectrum.cu:535,956)
  {
    double fb = z / c.zmax * (NZ - 1);
    double g = interp_mid(t.g, fb), fK = interp_mid(t.f_K, fb);
    double D1 = interp_mid(t.D1, fb), rs = interp_mid(t.r_sigma, fb);
    double ne = interp_mid(t.n_eff, fb), ncur = interp_mid(t.ncur, fb);
    double E = d_E(c, z);
    double W = (z < 1e-5) ? 0.0
                          : wq * 9. / 4. * H0_OVER_C * H0_OVER_C * H0_OVER_C * c.om * c.om * (1. + z) * (1. + z) *
                                g * g / E;
    double aa = 1. / (1 + z);
    double den = c.om + aa * (aa * aa * c.ow + (1. - c.om - c.ow));
    double om_m = c.om / den, om_v = c.ow * aa * aa * aa / den;
    double nsqr = ne * ne, w = c.w;
    double f1a = pow(om_m, -0.0732), f2a = pow(om_m, -0.1423), f3a = pow(om_m, 0.0725);
    double f1b = pow(om_m, -0.0307), f2b = pow(om_m, -0.0585), f3b = pow(om_m, 0.0743);
    double frac = om_v / (1. - om_m);
    double v[HC_COUNT];
    v[HC_W] = W;
    v[HC_INVFK] = 1.0 / fK;
    v[HC_RS] = rs;
    v[HC_D1SQ] = D1 * D1;
    v[HC_A] = pow(10.0, 1.5222 + 2.8553 * ne + 2.3706 * nsqr + 0.9903 * ne * nsqr + 0.2250 * nsqr * nsqr -
                            0.6038 * ncur + 0.1749 * om_v * (1.0 + w));
    v[HC_B] = pow(10.0, -0.5642 + 0.5864 * ne + 0.5716 * nsqr - 1.5474 * ncur + 0.2279 * om_v * (1.0 + w));
    v[HC_C] = pow(10.0, 0.3698 + 2.0404 * ne + 0.8161 * nsqr + 0.5869 * ncur);
    v[HC_GAM] = 0.1971 - 0.0843 * ne + 0.8460 * ncur;
    v[HC_ALPHA] = fabs(6.0835 + 1.3373 * ne - 0.1959 * nsqr - 5.5274 * ncur);
    v[HC_BETA] = 2.0379 - 0.7354 * ne + 0.3157 * nsqr + 1.2490 * ne * nsqr + 0.3980 * nsqr * nsqr - 0.1682 * ncur;
    v[HC_XNU] = pow(10.0, 5.2105 + 3.6902 * ne);
    v[HC_F1] = frac * f1b + (1 - frac) * f1a;
    v[HC_F2] = frac * f2b + (1 - frac) * f2a;
    v[HC_F3] = frac * f3b + (1 - frac) * f3a;
    v[HC_L2INVFK] = log2(1.0 / fK);
    v[HC_L2RS] = log2(rs);
    v[HC_L2F3C] = log2(v[HC_F3] * v[HC_C]);
    double* o = hcoef + (size_t)ci * HC_COUNT * NNODE;
    float* of = hcoef_f + (size_t)ci * HC_COUNT * NNODE;
    for (int q = 0; q < HC_COUNT; ++q) {
      o[q * NNODE + j] = v[q];
      of[q * NNODE + j] = (float)v[q];
    }
  }
}

// Halo-model node rows (trispectrum_integrand / pentaspectrum_integrand,
// halomodel.cu:392-496, their z-only factors) at the 96 line-of-sight nodes.
__global__ void k_halo_nodes(const CosmoDev* cos, const TablesDev* tab, int ci, HaloTab* halo) {
  const int j = threadIdx.x;
  if (j >= NNODE) return;
  const CosmoDev c = cos[ci];
  const TablesDev& t = tab[ci];
  const int i = j >> 1;
  const double cx = c.zmax / 2, dx = c.zmax / 2;
  const double z = (j & 1) ? cx + dx * c_gq_a[i] : cx - dx * c_gq_a[i];
  const double wq = c_gq_w[i] * dx;
  // linear interpolation on z_i = i z_max / (NZ - 1) (halomodel.cu:300-311)
  double f = z / c.zmax * (NZ - 1);
  int idx = (int)f;
  f -= idx;
  if (idx == NZ - 1) {
    idx = NZ - 2;
    f = 1.;
  }
  const double g = t.g[idx] * (1 - f) + t.g[idx + 1] * f;
  const double chi = t.f_K[idx] * (1 - f) + t.f_K[idx + 1] * f;
  const double D1 = t.D1[idx] * (1 - f) + t.D1[idx + 1] * f;
  const double aa = 1. / (1 + z);
  const double omz = c.om / (c.om + aa * (aa * aa * c.ow + (1. - c.om - c.ow)));  // om_m_of_z, bispectrum.cu:439-447
  const double dc = 1.686 * (1 + 0.0123 * log10(omz));
  const double pre = 1.5 * c.om / C_OVER_H0 / C_OVER_H0;
  const double los = wq * C_OVER_H0 / d_E(c, z);
  const double g2 = g * g, pre2 = pre * pre, zp2 = (1 + z) * (1 + z);
  double* h = halo->hn;
  h[HN_INVCHI * NNODE + j] = 1. / chi;
  h[HN_D1SQ * NNODE + j] = D1 * D1;
  h[HN_DC2 * NNODE + j] = dc * dc;
  h[HN_CZ * NNODE + j] = pow(1 + z, -1.01);
  h[HN_WTRI * NNODE + j] = los * g2 * g2 / (chi * chi) * pre2 * pre2 * zp2 * zp2;
  h[HN_WPEN * NNODE + j] = los * g2 * g2 * g2 / (chi * chi * chi * chi) * pre2 * pre2 * pre2 * zp2 * zp2 * zp2;
}

cudaError_t build_halo_nodes(const CosmoDev* d_cos, const TablesDev* d_tab, int ci, HaloTab* d_halo, cudaStream_t s) {
  k_halo_nodes<<<1, NNODE, 0, s>>>(d_cos, d_tab, ci, d_halo);
  return cudaGetLastError();
}

// Normalise the LOS weights of the FP32 node table by their maximum (kept in
// wscale) so that FP32 products stay far from the float range limits, and
// build the integrand constant blocks.
TP_TABLE_KERNEL k_finish(const CosmoDev* cos, const EHConst* eh, const TablesDev* tab, double* ncoef, float* ncoef_f,
                         float* fcoef_f, double* wscale64, double* wscale32, CosmoK<double>* ck64, CosmoK<float>* ck32,
                         int n) {
  int ci = blockIdx.x;
  if (ci >= n) return;
  __shared__ double wmax;
  if (threadIdx.x == 0) {
    double m = 0;
    const double* W = ncoef + (size_t)ci * NCP * NNODE + NC_W;
    for (int j = 0; j < NNODE; ++j) m = fmax(m, fabs(W[j * NCP]));
    wmax = m > 0 ? m : 1.0;
    wscale64[ci] = 1.0;
    wscale32[ci] = wmax;
    ck64[ci] = make_cosmok<double>(eh[ci], cos[ci], tab[ci].pk);
    CosmoK<float> k32 = make_cosmok<float>(eh[ci], cos[ci], tab[ci].pk);
    // log2(ell) range keeping every node's table coordinate
    // (log2 ell + log2(h/f_K) - PLT_LO) * INV at least 0.05 octaves (~1 cell)
    // inside the table
    double lo = -1e300, hi = 1e300;
    for (int j = 0; j < NNODE; ++j) {
      const double l2hf = ncoef[((size_t)ci * NNODE + j) * NCP + NC_L2HF];
      lo = fmax(lo, PLT_LO - l2hf + 0.05);
      hi = fmin(hi, PLT_HI - l2hf - 0.05);
    }
    k32.lgp_lo = (float)lo;
    k32.lgp_hi = (float)hi;
    ck32[ci] = k32;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < NNODE; j += blockDim.x) {
    size_t o = ((size_t)ci * NNODE + j) * NCP + NC_W;
    ncoef_f[o] = (float)(ncoef[o] / wmax);
    fcoef_f[(size_t)ci * NNODE * NCP + nf_index(j, NF_W)] = (float)(ncoef[o] / wmax);
  }
}

// log2 P_lin on the FP32 interpolation grid (log2(k h) uniform on [PLT_LO, PLT_HI])
// and its Catmull-Rom cubic per interval i: y(i + f) = y0 + f (c1 + f (c2 + f c3))
TP_TABLE_KERNEL k_plin_table(const CosmoDev* cos, const EHConst* eh, float4* plt, CosmoK<float>* ck32, int n) {
  // block b of a cosmology builds intervals [b * PLT_SLICE, (b + 1) * PLT_SLICE)
  constexpr int PLT_SLICE = 128;
  const int ci = blockIdx.x / (PLT_N / PLT_SLICE), a = (blockIdx.x % (PLT_N / PLT_SLICE)) * PLT_SLICE;
  if (ci >= n) return;
  const CosmoDev c = cos[ci];
  const EHConst e = eh[ci];
  // y[m] = log2 P at grid point m - 1, m = 0 .. PLT_N + 1; this slice needs
  // y[a .. a + PLT_SLICE + 3]
  __shared__ double y[PLT_SLICE + 4];
  for (int k = threadIdx.x; k < PLT_SLICE + 4; k += blockDim.x) {
    const int m = a + k;
    if (m > PLT_N + 1) continue;
    double kk = exp2(PLT_LO + (m - 1) * (PLT_HI - PLT_LO) / (PLT_N - 1));
    y[k] = log2(eh_linear_pk(e, kk / c.h));
  }
  __syncthreads();
  for (int u = threadIdx.x; u < PLT_SLICE; u += blockDim.x) {
    const int i = a + u;
    double ym1 = y[u], y0 = y[u + 1], y1 = y[u + 2], y2 = i + 3 < PLT_N + 2 ? y[u + 3] : y[u + 2];
    float4 q;
    q.x = (float)y0;
    q.y = (float)(0.5 * (y1 - ym1));
    q.z = (float)(0.5 * (2 * ym1 - 5 * y0 + 4 * y1 - y2));
    q.w = (float)(0.5 * (3 * (y0 - y1) + y2 - ym1));
    plt[(size_t)ci * PLT_N + i] = q;
  }
  if (a == 0 && threadIdx.x == 0 && !c.pk_given) ck32[ci].plt = (const float*)(plt + (size_t)ci * PLT_N);
}

// ---------------------------------------------------------------------------
void upload_gauss_nodes() {
  double a[48], w[48];
  gauss_legendre96(a, w);
  cudaMemcpyToSymbol(c_gq_a, a, sizeof(a));
  cudaMemcpyToSymbol(c_gq_w, w, sizeof(w));
}

cudaError_t build_tables(const CosmoDev* d_cos, EHConst* d_eh, const double* d_nz, int nz_stride, TablesDev* d_tab,
                         double* d_ncoef, float* d_ncoef_f, float* d_fcoef_f, double* d_hcoef, float* d_hcoef_f,
                         double* d_wscale64,
                         double* d_wscale32, CosmoK<double>* d_ck64, CosmoK<float>* d_ck32, float4* d_plt,
                         double* d_ehg, int n, cudaStream_t s) {
  // every launch is made of one-warp blocks (see above). An SM runs blocks of
  // different kernels together only in one shared-memory/L1 configuration:
  // these kernels ask for the one k_map3 runs in (maximum shared memory).
  static thread_local int carveout_set = -1;
  static thread_local size_t rsigma_smem = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (carveout_set != dev) {
    // k_rsigma (FP64-pipe bound) asks for shared memory it does not use: just
    // over half of what the resident k_map3<float> CTAs leave free on an SM,
    // so that one k_rsigma warp runs beside them instead of four (one per
    // sub-partition by registers) and contends less with k_map3's own FP64
    // instructions; alone it still fills the SM
    size_t used = 0;
    int smem_sm = 0, reserved = 0;
    if (map3_f32_resident_smem(&used) == cudaSuccess &&
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess) {
      const long free_b = (long)smem_sm - (long)used;
      rsigma_smem = free_b >= 2L * reserved + 2 ? (size_t)(free_b / 2 + 1) : 0;
      if (rsigma_smem > 48 * 1024) rsigma_smem = 48 * 1024;
    }
    cudaGetLastError();  // a failed query leaves rsigma_smem = 0
    const void* ks[] = {(const void*)k_eh_table, (const void*)k_norm, (const void*)k_fk, (const void*)k_g, (const void*)k_growth,
                        (const void*)k_rsigma, (const void*)k_node_coefs, (const void*)k_finish,
                        (const void*)k_plin_table};
    for (const void* k : ks)
      cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    carveout_set = dev;
  }
  k_eh_table<<<(unsigned)((long)n * EHG_N / 32), 32, 0, s>>>(d_cos, d_eh, d_ehg, n);
  k_norm<<<n, 32, 0, s>>>(d_cos, d_eh, d_tab, n);
  k_fk<<<n * (NZ / 32), 32, 0, s>>>(d_cos, d_tab, n);
  k_g<<<n * (NZ / 32), 32, 0, s>>>(d_cos, d_nz, nz_stride, d_tab, n);
  k_growth<<<n * (NZ / 32), 32, 0, s>>>(d_cos, d_tab, n);
  k_rsigma<<<(unsigned)((long)n * (NZ / RS_BINS)), 32, rsigma_smem, s>>>(d_cos, d_eh, d_tab, d_ehg, n);
  k_node_coefs<<<n * (NNODE / 32), 32, 0, s>>>(d_cos, d_tab, d_ncoef, d_ncoef_f, d_fcoef_f, d_hcoef, d_hcoef_f, n);
  k_finish<<<n, 32, 0, s>>>(d_cos, d_eh, d_tab, d_ncoef, d_ncoef_f, d_fcoef_f, d_wscale64, d_wscale32, d_ck64, d_ck32,
                            n);
  k_plin_table<<<n * (PLT_N / 128), 32, 0, s>>>(d_cos, d_eh, d_plt, d_ck32, n);
  return cudaGetLastError();
}

}  // namespace tp
