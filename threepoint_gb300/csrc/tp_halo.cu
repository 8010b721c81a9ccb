// Halo-model <Map^3> covariance terms T5, T6, T7.
//
// Reference (cuda_version/): halomodel.cu (sigma2 / dSigma2dm tables :179-276,
// get_sigma2 / get_dSigma2dm :279-375, hmf :31-59, SiCi :61-105, r_200
// :107-119, u_NFW :121-140, concentration :142-152, trispectrum_integrand /
// pentaspectrum_integrand and their 96-node line-of-sight integrals
// :392-510) and apertureStatisticsCovariance.cu (T5 / T6 / T7 :1199-1313,
// integrand_T5_infinite, integrand_T6_square / _rectangle,
// integrand_T7_infinite :2151-2314).
//
// Every term is one adaptive integral on the device engine over ln ell,
// angles and the halo mass m (linear in [1e9, 1e17] Msun/h). The inner
// line-of-sight sums are split into node chunks that the engine spreads over
// the CTA's threads. The mass tables sigma^2(m), dsigma^2/dm at z = 0 are
// 256 one-dimensional adaptive integrals per cosmology on the same engine.
#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tp_cov.cuh"
#include "tp_halo.h"
#include "tp_tables.cuh"

namespace tp {

namespace {

// ---------------------------------------------------------------------------
// sigma^2(m) and dsigma^2/dm at z = 0 (halomodel.cu:179-276): job i < NM is
// sigma^2(m_i), job NM + i is dsigma^2/dm(m_i); k in [0, 1e12] h/Mpc at
// relative 1e-4. The reference's host linear_pk is Eisenstein & Hu here
// whatever P(k) was given (its Pk_given global is never set).
__device__ inline double tophat_w(double x) { return 3.0 / (x * x * x) * (sin(x) - x * cos(x)); }
__device__ inline double tophat_dw(double x) {
  return (3 * (x * x - 3) * sin(x) + 9 * x * cos(x)) / x / x / x / x;
}

struct SigmaPol {
  static constexpr int G = 1, PD = 1, NS = 1, CH = 8, MINB = 1;
  static constexpr bool CLUSTER16 = false;
  __device__ static int slot(int) { return 0; }
  struct Rec {
    double v;
  };
  static constexpr int REC = (int)sizeof(Rec);
  static constexpr size_t PSMEM = 16;
  const int* job_order = nullptr;

  EHConst eh;  // norm^2 folded in
  double rhobar;
  double* out;  // [2 NM]
  int* status;
  double R, dR;
  int deriv, loaded;

  __device__ void begin_job(int job, char*, double* xmin, double* xmax) {
    const int i = job % NM;
    deriv = job / NM;
    const double m = pow(10., LOGM_MIN + i * ((LOGM_MAX - LOGM_MIN) / NM));
    R = pow(0.75 / PI * m / rhobar, 1. / 3.);
    dR = pow(0.75 / PI / rhobar, 1. / 3.) * pow(m, -2. / 3.) / 3.;
    xmin[0] = 0;
    xmax[0] = 1e12;
  }
  __device__ bool is_live(const char*) const { return false; }
  __device__ bool setup(int, const double* x, char* recp) {
    const double k = x[0];
    const double W = tophat_w(k * R);
    const double P = eh_linear_pk(eh, k);
    ((Rec*)recp)->v = deriv ? k * k * W * tophat_dw(k * R) * dR * P * k : k * k * W * W * P;
    return false;
  }
  __device__ void group(const char*, int, double* pv) { pv[0] = 0; }
  __device__ void finalize(const char* recp, const double*, double* fv) { fv[0] = ((const Rec*)recp)->v; }
  __device__ void end_job(int job, const double* V, const double*, long long, int st) {
    if (threadIdx.x == 0) {
      out[job] = V[0] / (deriv ? PI * PI : 2 * PI * PI);
      if (status) status[job] = st;
    }
  }
};

// FP32 copy of the node rows, the two weight rows scaled by their maximum
__global__ void k_halo_rows_f32(HaloTab* t) {
  const int j = threadIdx.x;
  if (j >= NNODE) return;
  double wmax[2] = {0, 0};
  for (int k = 0; k < NNODE; ++k) {
    wmax[0] = fmax(wmax[0], fabs(t->hn[HN_WTRI * NNODE + k]));
    wmax[1] = fmax(wmax[1], fabs(t->hn[HN_WPEN * NNODE + k]));
  }
  for (int r = 0; r < HN_COUNT; ++r) {
    double v = t->hn[r * NNODE + j];
    if (r == HN_WTRI) v /= wmax[0];
    if (r == HN_WPEN) v /= wmax[1];
    t->hnf[r * NNODE + j] = (float)v;
  }
  if (j == 0) {
    t->wmax[0] = wmax[0];
    t->wmax[1] = wmax[1];
  }
}

__global__ void k_halo_copy_tables(const double* src, HaloTab* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NM) {
    dst->sig2[i] = src[i];
    dst->dsig2[i] = src[NM + i];
  }
}

// ---------------------------------------------------------------------------
// Si and Ci (halomodel.cu:61-105): the reference's rational approximations
// (Rowe et al. 2015, GalSim, appendix B). Below 4: x P(x^2)/Q(x^2) and
// gamma + ln x + x^2 P'(x^2)/Q'(x^2); from 4 on the auxiliary functions
// f = F(y)/(x G(y)), g = F'(y)/(x^2 G'(y)), y = 1/x^2, with
// Si = pi/2 - f cos x - g sin x, Ci = f sin x - g cos x. Polynomials in
// Horner form.
template <typename R>
__device__ __forceinline__ R horner(const R* c, int n, R y) {
  R s = c[n - 1];
  for (int i = n - 2; i >= 0; --i) s = s * y + c[i];
  return s;
}

#define TP_SICI_SA                                                                                               \
  1, -4.54393409816329991e-2, 1.15457225751016682e-3, -1.41018536821330254e-5, 9.43280809438713025e-8,           \
      -3.53201978997168357e-10, 7.08240282274875911e-13, -6.05338212010422477e-16
#define TP_SICI_SB                                                                                              \
  1, 1.01162145739225565e-2, 4.99175116169755106e-5, 1.55654986308745614e-7, 3.28067571055789734e-10,          \
      4.5049097575386581e-13, 3.21107051193712168e-16
#define TP_SICI_CA                                                                                              \
  -0.25, 7.51851524438898291e-3, -1.27528342240267686e-4, 1.05297363846239184e-6, -4.68889508144848019e-9,      \
      1.06480802891189243e-11, -9.93728488857585407e-15
#define TP_SICI_CB                                                                                              \
  1, 1.1592605689110735e-2, 6.72126800814254432e-5, 2.55533277086129636e-7, 6.97071295760958946e-10,            \
      1.38536352772778619e-12, 1.89106054713059759e-15, 1.39759616731376855e-18
#define TP_SICI_FA                                                                                              \
  1, 7.44437068161936700618e2, 1.96396372895146869801e5, 2.37750310125431834034e7, 1.43073403821274636888e9,    \
      4.33736238870432522765e10, 6.40533830574022022911e11, 4.20968180571076940208e12, 1.00795182980368574617e13, \
      4.94816688199951963482e12, -4.94701168645415959931e11
#define TP_SICI_FB                                                                                              \
  1, 7.46437068161927678031e2, 1.97865247031583951450e5, 2.41535670165126845144e7, 1.47478952192985464958e9,    \
      4.58595115847765779830e10, 7.08501308149515401563e11, 5.06084464593475076774e12, 1.43468549171581016479e13, \
      1.11535493509914254097e13
#define TP_SICI_GA                                                                                              \
  1, 8.1359520115168615e2, 2.35239181626478200e5, 3.12557570795778731e7, 2.06297595146763354e9,                 \
      6.83052205423625007e10, 1.09049528450362786e12, 7.57664583257834349e12, 1.81004487464664575e13,           \
      6.43291613143049485e12, -1.36517137670871689e12
#define TP_SICI_GB                                                                                              \
  1, 8.19595201151451564e2, 2.40036752835578777e5, 3.26026661647090822e7, 2.23355543278099360e9,                \
      7.87465017341829930e10, 1.39866710696414565e12, 1.17164723371736605e13, 4.01839087307656620e13,           \
      3.99653257887490811e13

template <typename R>
struct SiCiCoef {
  // x < 4
  R sa[8], sb[7], ca[7], cb[8];
  // x >= 4
  R fa[11], fb[10], ga[11], gb[10];
};
__constant__ SiCiCoef<double> c_sici = {{TP_SICI_SA}, {TP_SICI_SB}, {TP_SICI_CA}, {TP_SICI_CB},
                                        {TP_SICI_FA}, {TP_SICI_FB}, {TP_SICI_GA}, {TP_SICI_GB}};
__constant__ SiCiCoef<float> c_sicif = {{TP_SICI_SA}, {TP_SICI_SB}, {TP_SICI_CA}, {TP_SICI_CB},
                                        {TP_SICI_FA}, {TP_SICI_FB}, {TP_SICI_GA}, {TP_SICI_GB}};

constexpr double EULER_GAMMA = 0.5772156649;  // the value halomodel.cu:83 uses

// Short FP32 node arithmetic (TP_HALO_FAST_FP32, default on): sin and cos of
// x >= 0 by reduction to r in [-pi/4, pi/4], x = r + k pi/2 with k = rint(2x/pi)
// and a three-constant FMA split of pi/2 (Cody & Waite), then the Taylor
// polynomials of sin (to r^9) and cos (to r^8), whose truncation errors on
// [-pi/4, pi/4] are below 2e-9 and 3e-8, and the quadrant's swap and signs:
// absolute error ~1e-7, as the library sincosf of an FP32 argument, in ~20
// instructions; quotients as reciprocal times numerator (2 ulp); ln on the SFU.
#ifndef TP_HALO_FAST_FP32
#define TP_HALO_FAST_FP32 1
#endif
#ifndef TP_HALO_F32_CH
#define TP_HALO_F32_CH 1
#endif
#ifndef TP_HALO_F32_MINB
#define TP_HALO_F32_MINB 3
#endif
__device__ __forceinline__ void sincos_r(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_r(float x, float* s, float* c) {
#if TP_HALO_FAST_FP32
  const float k = rintf(x * 0.636619772367581343f);  // 2 / pi
  float r = fmaf(-k, 1.57079637050628662f, x);        // pi/2 rounded to FP32
  r = fmaf(-k, -4.37113882867379317e-8f, r);          // next FP32 part of pi/2
  r = fmaf(-k, -1.77635684e-15f, r);                  // remainder
  const float r2 = r * r;
  // sin r = r (1 - r^2/3! + r^4/5! - r^6/7! + r^8/9!), cos r = 1 - r^2/2! + ... + r^8/8!
  float sp = fmaf(r2, 2.75573192e-6f, -1.98412698e-4f);
  sp = fmaf(sp, r2, 8.33333333e-3f);
  sp = fmaf(sp, r2, -1.66666667e-1f);
  const float sr = fmaf(sp * r2, r, r);
  float cp = fmaf(r2, 2.48015873e-5f, -1.38888889e-3f);
  cp = fmaf(cp, r2, 4.16666667e-2f);
  cp = fmaf(cp, r2, -0.5f);
  const float cr = fmaf(cp, r2, 1.0f);
  const int q = (int)k & 3;  // x = r + q pi/2 (mod 2 pi)
  const float sv = (q & 1) ? cr : sr, cv = (q & 1) ? sr : cr;
  *s = (q & 2) ? -sv : sv;
  *c = ((q + 1) & 2) ? -cv : cv;
#else
  sincosf(x, s, c);
#endif
}
__device__ __forceinline__ double log_r(double x) { return log(x); }
__device__ __forceinline__ float log_r(float x) {
#if TP_HALO_FAST_FP32
  return __logf(x);
#else
  return logf(x);
#endif
}
__device__ __forceinline__ double div_r(double a, double b) { return a / b; }
__device__ __forceinline__ float div_r(float a, float b) {
#if TP_HALO_FAST_FP32
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

template <typename R>
__device__ __forceinline__ const SiCiCoef<R>& sici_coef() {
  if constexpr (sizeof(R) == 8) return c_sici;
  else return c_sicif;
}

// Si(x) / x and (Ci(x) - gamma - ln x) / x^2 for x < 4
template <typename R>
__device__ __forceinline__ void sici_small(R x2, R& si_over_x, R& ci_rest_over_x2) {
  const SiCiCoef<R>& k = sici_coef<R>();
  si_over_x = div_r(horner(k.sa, 8, x2), horner(k.sb, 7, x2));
  ci_rest_over_x2 = div_r(horner(k.ca, 7, x2), horner(k.cb, 8, x2));
}
// f(x), g(x) for x >= 4
template <typename R>
__device__ __forceinline__ void sici_fg(R x, R& f, R& g) {
  const SiCiCoef<R>& k = sici_coef<R>();
  const R y = div_r((R)1, x * x);
  f = div_r(horner(k.fa, 11, y), horner(k.fb, 10, y) * x);
  g = div_r(horner(k.ga, 11, y) * y, horner(k.gb, 10, y));
}



// Truncated NFW profile in Fourier space times F(c) = ln(1+c) - c/(1+c)
// (u_NFW, halomodel.cu:121-140), with arg1 = k r_200 / c, arg2 = arg1 (1+c):
//   sin(arg1) (Si(arg2) - Si(arg1)) + cos(arg1) (Ci(arg2) - Ci(arg1)) - sin(arg1 c) / arg2.
// The differences are formed without the large common parts: from 4 on
// Si(b) - Si(a) = (f_a cos a + g_a sin a) - (f_b cos b + g_b sin b); below 4 on
// both sides Ci(b) - Ci(a) = ln(1+c) + b^2 r(b) - a^2 r(a); and
// sin(arg1 c) = sin(arg2 - arg1) = sin(arg2) cos(arg1) - cos(arg2) sin(arg1).
// In FP32 this keeps u accurate to ~1e-6 where the reference's direct
// differences of Si and Ci (each near pi/2 or 0 for large arguments) would
// lose every digit.
template <typename R>
__device__ __forceinline__ R u_nfw_f(R a1, R opc, R lnopc) {
  const R a2 = a1 * opc;
  R s1, c1, s2, c2;
  sincos_r(a1, &s1, &c1);
  sincos_r(a2, &s2, &c2);
  R dsi, dci;
  if (a2 < (R)4) {
    R q1, r1, q2, r2;
    sici_small<R>(a1 * a1, q1, r1);
    sici_small<R>(a2 * a2, q2, r2);
    dsi = a2 * q2 - a1 * q1;
    dci = lnopc + a2 * a2 * r2 - a1 * a1 * r1;
  } else if (a1 < (R)4) {
    R q1, r1, f2, g2;
    sici_small<R>(a1 * a1, q1, r1);
    sici_fg<R>(a2, f2, g2);
    dsi = ((R)(0.5 * PI) - f2 * c2 - g2 * s2) - a1 * q1;
    dci = (f2 * s2 - g2 * c2) - ((R)EULER_GAMMA + log_r(a1) + a1 * a1 * r1);
  } else {
    R f1, g1, f2, g2;
    sici_fg<R>(a1, f1, g1);
    sici_fg<R>(a2, f2, g2);
    dsi = (f1 * c1 + g1 * s1) - (f2 * c2 + g2 * s2);
    dci = (f2 * s2 - g2 * c2) - (f1 * s1 - g1 * c1);
  }
  const R s12 = s2 * c1 - c2 * s1;  // sin(a2 - a1)
  return s1 * dsi + c1 * dci - div_r(s12, a2);
}

// ---------------------------------------------------------------------------
// T5 (6-D: ln l1, ln l2, ln l5, phi1, phi2, m), T6 (7-D: ln l3, ln l4, ln l5,
// phi3, phi4, phi5, m), T7 (7-D: ln l1, ln l2, ln l4, ln l5, phi1, phi2, m).
template <int KIND, typename R = double>
struct HaloProd {
  static constexpr int DIM = KIND == 5 ? 6 : 7;
  static constexpr int NL = KIND == 7 ? 6 : 4;  // ell arguments of the tri-/pentaspectrum
  static constexpr int NCH = 8;                 // node chunks of 12
  static constexpr int G = KIND == 5 ? 2 * NCH : NCH;
  static constexpr int PD = 1;
  static constexpr int NS = KIND == 5 ? 2 : 1;
  __device__ static int slot(int g) { return KIND == 5 ? (g >= NCH ? 1 : 0) : 0; }
  // regions per chunk and CTAs per SM: the FP32 form takes one region per
  // chunk (half the point records and partial sums in shared memory) so that
  // three CTAs fit on an SM
  static constexpr int CH = sizeof(R) == 4 ? TP_HALO_F32_CH : 2;
  static constexpr int MINB = sizeof(R) == 4 ? TP_HALO_F32_MINB : 2;
  static constexpr bool CLUSTER16 = true;
  struct Rec {
    R l[NL];
    double pm;    // -rhobar/m dsig2/sig2 A (m/rhobar)^n (x the weight scale in FP32): the mass-function factor
    R s2m;        // sigma^2(m) at z = 0
    R cm;         // mass part of the concentration, 10.14 (m / 2e12)^-0.081
    R r200;       // r_200(m)
    double wt;    // filter product, ell factors and window
    R pell, pl2;  // T5: ell_1 and log2 ell_1 of P(ell_1)
    int valid, los;
  };
  static constexpr int REC = (int)sizeof(Rec);
  const int* job_order = nullptr;
  static constexpr size_t PSMEM = sizeof(R) * HN_COUNT * NNODE + (KIND == 5 ? sizeof(R) * HC_COUNT * NNODE : 0) + 64;

  const CovJob* jobs;
  const HaloTab* halo;     // this cosmology's halo tables (global)
  const R* hcoef;          // T5: Halofit node rows of P(ell)
  CosmoK<R> ck;
  double rhobar;
  double psn;              // shape-noise power of P(ell)
  int constant_ps;
  double thetaMax, thetaMaxY;
  double norm;
  double* out;
  int* status;
  R* s_hn;
  R* s_hc;
  double th[6], lmax;
  int loaded;

  // node tables into shared memory (all threads of the CTA)
  __device__ void load_tables(char* psmem) {
    s_hn = (R*)psmem;
    s_hc = s_hn + HN_COUNT * NNODE;
    __syncthreads();
    const R* hn = sizeof(R) == 8 ? (const R*)(const void*)halo->hn : (const R*)(const void*)halo->hnf;
    for (int i = threadIdx.x; i < HN_COUNT * NNODE; i += blockDim.x) s_hn[i] = hn[i];
    if (KIND == 5)
      for (int i = threadIdx.x; i < HC_COUNT * NNODE; i += blockDim.x) s_hc[i] = hcoef[i];
    __syncthreads();
  }

  // mass-dependent factors of a point record
  __device__ void set_mass(Rec& r, double m) const {
    const double s2m = minterp(halo->sig2, m), ds2m = minterp(halo->dsig2, m);
    const double mr = m / rhobar;
    double mn = mr * mr * mr * mr;
    if (NL == 6) mn *= mr * mr;
    r.pm = -rhobar / m * ds2m / s2m * 0.322 * mn;
    if (sizeof(R) == 4) r.pm *= halo->wmax[NL == 6 ? 1 : 0];
    r.s2m = (R)s2m;
    r.cm = (R)(10.14 * pow(m / 2e12, -0.081));
    r.r200 = (R)pow(0.75 / PI * mr / 200, 1. / 3.);
  }

  __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) {
    if (!loaded) {
      load_tables(psmem);
      loaded = 1;
    }
    const CovJob& J = jobs[job];
    for (int i = 0; i < 6; ++i) th[i] = J.th[i];
    lmax = J.lmax;
    const double ll = log(J.lmin), lh = log(lmax);
    const int nlog = KIND == 7 ? 4 : 3;
    for (int d = 0; d < nlog; ++d) {
      xmin[d] = ll;
      xmax[d] = lh;
    }
    for (int d = nlog; d < DIM - 1; ++d) {
      xmin[d] = 0;
      xmax[d] = 2 * PI;
    }
    xmin[DIM - 1] = pow(10., LOGM_MIN);
    xmax[DIM - 1] = pow(10., LOGM_MAX);
  }

  __device__ bool is_live(const char* r) const { return ((const Rec*)r)->valid != 0; }

  // mass-table lookup (halomodel.cu:279-299): the index runs over NM - 1
  // intervals of [LOGM_MIN, LOGM_MAX] although the table holds NM masses
  // spaced by (LOGM_MAX - LOGM_MIN) / NM
  __device__ static double minterp(const double* arr, double m) {
    double f = (log10(m) - LOGM_MIN) / (LOGM_MAX - LOGM_MIN) * (NM - 1);
    int idx = (int)f;
    f -= idx;
    if (idx >= NM - 1) {
      idx = NM - 2;
      f = 1.;
    }
    if (idx < 0) {
      idx = 0;
      f = 0.;
    }
    return arr[idx] * (1 - f) + arr[idx + 1] * f;
  }

  __device__ bool setup(int p, const double* x, char* recp) {
    (void)p;
    Rec& r = *(Rec*)recp;
    double wt = 0, m = x[DIM - 1];
    bool ok = false;
    if constexpr (KIND == 5) {
      const double l1 = exp(x[0]), l2 = exp(x[1]), l5 = exp(x[2]);
      const double s3 = l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(x[3]);
      const double s6 = l1 * l1 + l5 * l5 + 2 * l1 * l5 * cos(x[4]);
      if (s3 > 0 && s6 > 0) {
        const double l3 = sqrt(s3), l6 = sqrt(s6);
        if (!(l3 > lmax || l6 > lmax)) {
          const double lp = l1 * l2 * l5;
          wt = uhat(l1 * th[0]) * uhat(l2 * th[1]) * uhat(l3 * th[2]) * uhat(l1 * th[3]) * uhat(l5 * th[4]) *
               uhat(l6 * th[5]) * lp * lp;
          r.l[0] = (R)l2, r.l[1] = (R)l3, r.l[2] = (R)l5, r.l[3] = (R)l6;
          r.pell = (R)l1;
          r.pl2 = (R)log2(l1);
          ok = true;
        }
      }
    } else if constexpr (KIND == 6) {
      const double l3 = exp(x[0]), l4 = exp(x[1]), l5 = exp(x[2]);
      const double p3 = x[3], p4 = x[4], p5 = x[5];
      double s6 = l3 * l3 + l4 * l4 + l5 * l5 + 2 * (l3 * l4 * cos(p3 - p4) - l3 * l5 * cos(p3 - p5) - l4 * l5 * cos(p4 - p5));
      const double l6 = s6 > 0 ? sqrt(s6) : 0.0;
      if (l6 > 0 && !(l6 > lmax)) {
        double sp, cp;
        sincos(p3, &sp, &cp);
        const double G = g_square<double>(thetaMax, thetaMaxY, l3 * cp, l3 * sp);
        const double lp = l3 * l4 * l5;
        wt = uhat(l3 * th[2]) * uhat(l4 * th[3]) * uhat(l5 * th[4]) * uhat(l6 * th[5]) * lp * lp * G;
        r.l[0] = (R)l3, r.l[1] = (R)l4, r.l[2] = (R)l5, r.l[3] = (R)l6;
        ok = true;
      }
    } else {
      const double l1 = exp(x[0]), l2 = exp(x[1]), l4 = exp(x[2]), l5 = exp(x[3]);
      const double s3 = l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(x[4]);
      const double s6 = l4 * l4 + l5 * l5 + 2 * l4 * l5 * cos(x[5]);
      if (s3 > 0 && s6 > 0) {
        const double l3 = sqrt(s3), l6 = sqrt(s6);
        const double lp = l1 * l2 * l4 * l5;
        wt = uhat(l1 * th[0]) * uhat(l2 * th[1]) * uhat(l3 * th[2]) * uhat(l4 * th[3]) * uhat(l5 * th[4]) *
             uhat(l6 * th[5]) * lp * lp;
        r.l[0] = (R)l1, r.l[1] = (R)l2, r.l[2] = (R)l3, r.l[3] = (R)l4, r.l[4] = (R)l5, r.l[5] = (R)l6;
        ok = true;
      }
    }
    r.valid = ok && wt != 0.0;
    r.wt = wt;
    if (r.valid) set_mass(r, m);
    r.los = r.valid && (KIND != 5 || !constant_ps);
    return r.valid;
  }

  __device__ void group(const char* recp, int g, double* pv) {
    typedef Mth<R> M;
    const Rec& r = *(const Rec*)recp;
    if (KIND == 5 && g < NCH) {
      // P(ell_1) node chunk
      KSum<R> acc;
      if (r.los) {
        const int j0 = g * (NNODE / NCH);
        for (int j = j0; j < j0 + NNODE / NCH; ++j) {
          R v = pell_node<R>(s_hc, j, r.pell, r.pl2, ck);
          if (v != v) v = 0;
          acc.add(v);
        }
      }
      pv[0] = (double)acc.s;
      return;
    }
    const int ch = KIND == 5 ? g - NCH : g;
    const int j0 = ch * (NNODE / NCH);
    const R q = (R)0.707, p = (R)0.3;
    KSum<R> acc;
    for (int j = j0; j < j0 + NNODE / NCH; ++j) {
      const R invchi = s_hn[HN_INVCHI * NNODE + j];
      // Sheth-Tormen multiplicity at nu = delta_c^2 / sigma^2(m, z)
      const R qnu = q * s_hn[HN_DC2 * NNODE + j] / (r.s2m * s_hn[HN_D1SQ * NNODE + j]);
      R fnu;
      if constexpr (sizeof(R) == 8)
        fnu = (1 + pow(qnu, -p)) * sqrt(qnu / (2 * PI)) * exp(-0.5 * qnu);
      else
        fnu = (1.f + M::ex2(-p * M::lg2(qnu))) * sqrtf(qnu * (float)(0.5 / PI)) *
              M::ex2(qnu * (float)(-0.5 / LN2));
      // NFW: concentration, F(c), scale k -> arg1 = k r_200 / c
      const R c = r.cm * s_hn[HN_CZ * NNODE + j];
      const R opc = 1 + c;
      const R lnopc = log_r(opc);
      const R invF = div_r((R)1, lnopc - div_r(c, opc));
      const R a = r.r200 / c * invchi;
      R prod = fnu * s_hn[(NL == 6 ? HN_WPEN : HN_WTRI) * NNODE + j];
#pragma unroll
      for (int i = 0; i < NL; ++i) prod *= u_nfw_f<R>(r.l[i] * a, opc, lnopc) * invF;
      acc.add(prod);
    }
    pv[0] = (double)acc.s;
  }

  __device__ void finalize(const char* recp, const double* sum, double* fv) {
    const Rec& r = *(const Rec*)recp;
    if (!r.valid) {
      fv[0] = 0;
      return;
    }
    double v = r.wt * r.pm;
    if (KIND == 5) v *= ((r.los ? sum[0] : 0.0) + psn) * sum[1];
    else v *= sum[0];
    fv[0] = v;
  }

  __device__ void end_job(int job, const double* V, const double*, long long, int st) {
    if (threadIdx.x == 0) {
      out[job] = V[0] * norm;
      if (status) status[job] = st;
    }
  }
};

// Integrand values of term KIND at points x (ndim = DIM): setup, every node
// chunk and the final product as the engine forms them, one thread per point.
template <int KIND, typename R>
__global__ void k_halo_points(HaloProd<KIND, R> pol, const double* x, long n, double* out) {
  extern __shared__ __align__(16) char psmem[];
  pol.load_tables(psmem);
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  typedef HaloProd<KIND, R> P;
  typename P::Rec r;
  double s[2] = {0, 0}, f;
  if (pol.setup(0, x + i * P::DIM, (char*)&r))
    for (int g = 0; g < P::G; ++g) {
      double v;
      pol.group((const char*)&r, g, &v);
      s[P::slot(g)] += v;
    }
  pol.finalize((const char*)&r, s, &f);
  out[i] = f;
}

// One-halo line-of-sight trispectrum (l1..l4) and pentaspectrum (l1..l6) at
// rows (m, l1, ..., l6): trispectrum_limber_integrated /
// pentaspectrum_limber_integrated over [0, z_max] (halomodel.cu:430-510).
template <typename R>
__global__ void k_halo_los(HaloProd<6, R> tri, HaloProd<7, R> pen, const double* pts, long n, double* otri,
                           double* open) {
  extern __shared__ __align__(16) char psmem[];
  tri.load_tables(psmem);
  pen.s_hn = tri.s_hn;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pts + 7 * i;
  typename HaloProd<6, R>::Rec rt;
  typename HaloProd<7, R>::Rec rp;
  tri.set_mass(rt, p[0]);
  pen.set_mass(rp, p[0]);
  for (int k = 0; k < 4; ++k) rt.l[k] = (R)p[1 + k];
  for (int k = 0; k < 6; ++k) rp.l[k] = (R)p[1 + k];
  double st = 0, sp = 0;
  for (int g = 0; g < HaloProd<6, R>::NCH; ++g) {
    double v;
    tri.group((const char*)&rt, g, &v);
    st += v;
    pen.group((const char*)&rp, g, &v);
    sp += v;
  }
  otri[i] = st * rt.pm;
  open[i] = sp * rp.pm;
}

}  // namespace

// Builds the halo-model tables of one cosmology on first use.
int ensure_halo(tp_ctx* ctx, int cosmo) {
  if ((int)ctx->halo_ready.size() > cosmo && ctx->halo_ready[cosmo]) return TP_OK;
  cudaError_t e = cudaSuccess;
  if (!ctx->d_halo) {
    e = cudaMalloc(&ctx->d_halo, sizeof(HaloTab) * (size_t)ctx->cosmo_cap);
    if (e != cudaSuccess) {
      ctx->d_halo = nullptr;
      return tp_cuda(ctx, e, "halo tables");
    }
  }
  if ((int)ctx->halo_ready.size() < ctx->cosmo_cap) ctx->halo_ready.resize(ctx->cosmo_cap, 0);
  HaloTab* tab = ctx->d_halo + cosmo;
  const size_t o_s = (sizeof(double) * 2 * NM + 255) & ~size_t(255);
  int st = ctx->ensure_io(o_s + sizeof(int) * 2 * NM + 256);
  if (st) return st;
  char* b = ctx->d_io;
  SigmaPol pol;
  memset(&pol, 0, sizeof(pol));
  e = cudaMemcpyAsync(&pol.eh, ctx->d_eh + cosmo, sizeof(EHConst), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "halo constants");
  pol.rhobar = RHO_CRIT * ctx->h_cos[cosmo].om;
  pol.out = (double*)b;
  pol.status = (int*)(b + o_s);
  st = run_engine<1>(ctx, pol, 2 * NM, 1e-4, 1);
  if (st) return st;
  std::vector<int> hs(2 * NM);
  e = cudaMemcpy(hs.data(), b + o_s, sizeof(int) * 2 * NM, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "halo tables");
  for (int v : hs)
    if (v) return tp_fail(ctx, TP_ERR_CAPACITY, "sigma^2(m) table integral hit the region cap");
  k_halo_copy_tables<<<1, NM, 0, ctx->stream>>>((const double*)b, tab);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = build_halo_nodes(ctx->d_cos, ctx->d_tab, cosmo, tab, ctx->stream);
  if (e == cudaSuccess) {
    k_halo_rows_f32<<<1, NNODE, 0, ctx->stream>>>(tab);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "halo tables");
  ctx->halo_ready[cosmo] = 1;
  return TP_OK;
}

namespace {

// policy parameters of cosmology cosmo (everything but the job list and outputs)
template <int KIND, typename R>
int halo_policy(tp_ctx* ctx, int cosmo, double theta_max, double theta_max_y, double norm, HaloProd<KIND, R>& pol) {
  memset(&pol, 0, sizeof(pol));
  pol.halo = ctx->d_halo + cosmo;
  pol.hcoef = (sizeof(R) == 8 ? (const R*)(const void*)ctx->d_hcoef : (const R*)(const void*)ctx->d_hcoef32) +
              (size_t)cosmo * HC_COUNT * NNODE;
  cudaError_t e = cudaMemcpyAsync(&pol.ck, (const char*)(sizeof(R) == 8 ? ctx->d_ck64 : ctx->d_ck32) + sizeof(CosmoK<R>) * cosmo,
                                  sizeof(CosmoK<R>), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "halo term constants");
  pol.rhobar = RHO_CRIT * ctx->h_cos[cosmo].om;
  pol.psn = 0.5 * ctx->sigma_eps * ctx->sigma_eps / ctx->ngal;
  pol.constant_ps = ctx->constant_ps;
  pol.thetaMax = theta_max;
  pol.thetaMaxY = theta_max_y;
  pol.norm = norm;
  return TP_OK;
}

template <int KIND, typename R>
int run_halo_kind(tp_ctx* ctx, int cosmo, const JobSet& js, double theta_max, double theta_max_y, double norm,
                  double rel_tol, std::vector<double>& res, int& bad) {
  res.assign(js.jobs.size(), 0.0);
  if (js.jobs.empty()) return TP_OK;
  HaloProd<KIND, R> pol;
  int st = halo_policy<KIND, R>(ctx, cosmo, theta_max, theta_max_y, norm, pol);
  if (st) return st;
  // one cluster of 8 CTAs per integral: a T5-T7 point costs 96 nodes x 4-6
  // NFW profiles, so a single integral (or the most expensive one of a batch)
  // spreads over 8 SMs; the region sequence is that of one CTA per integral
  // A batch too large for 16-CTA clusters runs a first pass that stops at the
  // context's region cap (32768 by default); the integrals that need more (the
  // smallest radii) continue in the escalation passes, a handful at a time on
  // 16-CTA clusters, instead of setting the batch's time on 8 CTAs.
  constexpr int D = HaloProd<KIND, R>::DIM;
  const bool big = ctx->halo_cluster == 16 &&
                   (long)js.jobs.size() * 16 > (long)engine_slots<D, HaloProd<KIND, R>>(ctx);
  return run_jobs<D>(ctx, pol, js.jobs, rel_tol, ctx->halo_cluster, res, bad, big ? ctx->region_cap : 0);
}

// the reference's tolerances of the T5, T6, T7 integrals (:1222, :1271, :1307)
double halo_tol(const tp_ctx* ctx, int term) {
  const double d = term == 5 ? 1e-2 : 1e-1;
  return ctx->cov_rel_tol[term] > 0 ? ctx->cov_rel_tol[term] : d;
}

}  // namespace

template <typename R>
static int halo_terms_t(tp_ctx* ctx, int cosmo, int term, int geom, double theta_max, double area,
                        const std::vector<std::array<double, 6>>& th6, std::vector<double>& out, int& bad) {
  const size_t n = th6.size();
  out.assign(n, 0.0);
  if (n == 0) return TP_OK;
  int st = ensure_halo(ctx, cosmo);
  if (st) return st;
  const double two_pi = 2 * PI;
  JobSet js;
  std::vector<int> id(n);
  for (size_t i = 0; i < n; ++i) {
    const double* t = th6[i].data();
    id[i] = js.add(t, 6, HALO_LMIN, halo_lmax(term, t));
  }
  std::vector<double> r;
  if (term == 5) {
    st = run_halo_kind<5, R>(ctx, cosmo, js, theta_max, theta_max, 1 / area / pow(two_pi, 5), halo_tol(ctx, 5), r, bad);
  } else if (term == 7) {
    st = run_halo_kind<7, R>(ctx, cosmo, js, theta_max, theta_max, 1 / area / pow(two_pi, 6), halo_tol(ctx, 7), r, bad);
  } else {
    const double tmy = geom == TP_GEOM_RECTANGLE ? ctx->theta_max_smaller : theta_max;
    st = run_halo_kind<6, R>(ctx, cosmo, js, theta_max, tmy, 1 / pow(two_pi, 6), halo_tol(ctx, 6), r, bad);
  }
  if (st) return st;
  for (size_t i = 0; i < n; ++i) out[i] = r[id[i]];
  return TP_OK;
}

int halo_terms(tp_ctx* ctx, int cosmo, int term, int geom, double theta_max, double area,
               const std::vector<std::array<double, 6>>& th6, int precision, std::vector<double>& out, int& bad) {
  return precision == TP_FP32 ? halo_terms_t<float>(ctx, cosmo, term, geom, theta_max, area, th6, out, bad)
                              : halo_terms_t<double>(ctx, cosmo, term, geom, theta_max, area, th6, out, bad);
}

double halo_lmax(int term, const double* t) {
  const double a = std::min({t[0], t[1], t[2]}), b = std::min({t[3], t[4], t[5]});
  return 10. / (term == 7 ? std::min(a, b) : std::max(a, b));
}

}  // namespace tp

using namespace tp;

static int check_halo_args(tp_ctx* ctx, int cosmo) {
  if (!ctx) return TP_ERR_ARG;
  if (cosmo < 0 || cosmo >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  cudaSetDevice(ctx->device);
  return ensure_halo(ctx, cosmo);
}

extern "C" int tp_halo_tables(tp_ctx* ctx, int cosmo, double* out) {
  if (!out) return TP_ERR_ARG;
  int st = check_halo_args(ctx, cosmo);
  if (st) return st;
  cudaError_t e = cudaMemcpy(out, ctx->d_halo[cosmo].sig2, sizeof(double) * NM, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(out + NM, ctx->d_halo[cosmo].dsig2, sizeof(double) * NM, cudaMemcpyDeviceToHost);
  return tp_cuda(ctx, e, "halo tables");
}

template <typename R>
static int halo_los_t(tp_ctx* ctx, int cosmo, const double* pts, long n, double* tri, double* penta) {
  HaloProd<6, R> tri_pol;
  HaloProd<7, R> pen_pol;
  int st = halo_policy<6, R>(ctx, cosmo, 0, 0, 1, tri_pol);
  if (!st) st = halo_policy<7, R>(ctx, cosmo, 0, 0, 1, pen_pol);
  if (st) return st;
  const size_t o_t = (sizeof(double) * 7 * n + 255) & ~size_t(255), o_p = o_t + ((sizeof(double) * n + 255) & ~size_t(255));
  st = ctx->ensure_io(o_p + sizeof(double) * n + 256);
  if (st) return st;
  char* b = ctx->d_io;
  cudaError_t e = cudaMemcpyAsync(b, pts, sizeof(double) * 7 * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    k_halo_los<R><<<(unsigned)((n + 63) / 64), 64, HaloProd<6, R>::PSMEM, ctx->stream>>>(
        tri_pol, pen_pol, (const double*)b, n, (double*)(b + o_t), (double*)(b + o_p));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(tri, b + o_t, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(penta, b + o_p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return tp_cuda(ctx, e, "halo line-of-sight points");
}

extern "C" int tp_halo_los(tp_ctx* ctx, int cosmo, const double* pts, long n, int precision, double* tri,
                           double* penta) {
  if (!pts || !tri || !penta || n < 0 || (precision != TP_FP64 && precision != TP_FP32)) return TP_ERR_ARG;
  int st = check_halo_args(ctx, cosmo);
  if (st) return st;
  if (n == 0) return TP_OK;
  for (long i = 0; i < n; ++i) {
    const double m = pts[7 * i];
    if (!(m >= 1e9 && m <= 1e17)) return tp_fail(ctx, TP_ERR_ARG, "halo mass outside [1e9, 1e17]");
    for (int k = 1; k < 7; ++k)
      if (!(pts[7 * i + k] > 0)) return tp_fail(ctx, TP_ERR_ARG, "ell must be > 0");
  }
  return precision == TP_FP32 ? halo_los_t<float>(ctx, cosmo, pts, n, tri, penta)
                              : halo_los_t<double>(ctx, cosmo, pts, n, tri, penta);
}

template <int KIND, typename R>
static int halo_points(tp_ctx* ctx, int cosmo, const double* th6, double lmax, double theta_max, double theta_max_y,
                       const double* x, long n, double* out) {
  typedef HaloProd<KIND, R> P;
  constexpr int D = P::DIM;
  P pol;
  int st = halo_policy<KIND, R>(ctx, cosmo, theta_max, theta_max_y, 1, pol);
  if (st) return st;
  for (int k = 0; k < 6; ++k) pol.th[k] = th6[k];
  pol.lmax = lmax;
  const size_t o_o = (sizeof(double) * D * n + 255) & ~size_t(255);
  st = ctx->ensure_io(o_o + sizeof(double) * n + 256);
  if (st) return st;
  char* b = ctx->d_io;
  cudaError_t e = cudaMemcpyAsync(b, x, sizeof(double) * D * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) {
    k_halo_points<KIND, R><<<(unsigned)((n + 63) / 64), 64, P::PSMEM, ctx->stream>>>(pol, (const double*)b, n,
                                                                                   (double*)(b + o_o));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, b + o_o, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return tp_cuda(ctx, e, "halo integrand points");
}

template <typename R>
static int halo_points_t(tp_ctx* ctx, int cosmo, int term, const double* th6, double lmax, double tm, double tmy,
                         const double* x, long n, double* out) {
  if (term == 5) return halo_points<5, R>(ctx, cosmo, th6, lmax, tm, tmy, x, n, out);
  if (term == 6) return halo_points<6, R>(ctx, cosmo, th6, lmax, tm, tmy, x, n, out);
  return halo_points<7, R>(ctx, cosmo, th6, lmax, tm, tmy, x, n, out);
}

extern "C" int tp_halo_integrand_points(tp_ctx* ctx, int cosmo, int term, int geometry, double theta_max,
                                        const double* th6, const double* x, long n, int precision, double* out) {
  if (!ctx || !th6 || !x || !out || n < 0 || term < 5 || term > 7) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (term == 6 && geometry != TP_GEOM_SQUARE && geometry != TP_GEOM_RECTANGLE)
    return tp_fail(ctx, TP_ERR_ARG, "T6: only coded for square and rectangular survey geometries");
  if (term == 6 && geometry == TP_GEOM_RECTANGLE && !(ctx->theta_max_smaller > 0))
    return tp_fail(ctx, TP_ERR_STATE, "rectangular geometry needs tp_set_rectangle_side");
  int st = check_halo_args(ctx, cosmo);
  if (st) return st;
  if (n == 0) return TP_OK;
  const int D = term == 5 ? 6 : 7;
  for (long i = 0; i < n; ++i) {
    const double m = x[D * i + D - 1];
    if (!(m >= 1e9 && m <= 1e17)) return tp_fail(ctx, TP_ERR_ARG, "halo mass outside [1e9, 1e17]");
  }
  const double lmax = halo_lmax(term, th6);
  const double tmy = geometry == TP_GEOM_RECTANGLE ? ctx->theta_max_smaller : theta_max;
  return precision == TP_FP32 ? halo_points_t<float>(ctx, cosmo, term, th6, lmax, theta_max, tmy, x, n, out)
                              : halo_points_t<double>(ctx, cosmo, term, th6, lmax, theta_max, tmy, x, n, out);
}

extern "C" int tp_ctx_set_halo_cluster(tp_ctx* ctx, int ctas) {
  if (!ctx || (ctas != 1 && ctas != 8 && ctas != 16)) return TP_ERR_ARG;
  ctx->halo_cluster = ctas;
  return TP_OK;
}

extern "C" int tp_ctx_set_cov_tolerance(tp_ctx* ctx, int term, double rel_tol) {
  if (!ctx || term < 5 || term > 7 || !(rel_tol >= 0)) return TP_ERR_ARG;
  ctx->cov_rel_tol[term] = rel_tol;
  return TP_OK;
}
