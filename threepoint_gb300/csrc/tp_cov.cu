// <Map^3> covariance terms T1, T2, T4 and the convergence power spectrum P(ell).
//
// Reference (cuda_version/apertureStatisticsCovariance.cu): G_circle/G_square
// (:117-153), T1_total/T2_total/T4_total (:272-683), T1/T2/T4 (:1065-1197),
// the integrand kernels integrand_T1_circle/_square/_infinite,
// integrand_T2_part1/_part2_circle/_part2_square and integrand_T4_infinite
// (:1886-2149); Pell / GQ96_of_Pk / limber_integrand_power_spectrum /
// P_k_nonlinear (cuda_version/bispectrum.cu:511-600,935-991).
//
// Every term T(theta1..theta6) is one adaptive integral on the device engine;
// a batch of covariance entries is expanded host-side into its permutation
// terms (the reference's multiplicity tables), duplicates are merged, all
// distinct integrals of one kind run in one persistent launch, and the
// totals are reassembled. P(ell) is a 96-node line-of-sight sum of the revised
// Halofit spectrum with the T17 correction; a point needing several P(ell)
// splits them into (P index x node group) items.
#include <cuda_runtime.h>

#include <type_traits>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "tp_bispec.cuh"
#include "tp_capi_internal.h"
#include "tp_cov.cuh"
#include "tp_cubature.cuh"
#include "tp_halo.h"
#include "tp_internal.cuh"
#include "tp_kernels.cuh"

namespace tp {

// ---------------------------------------------------------------------------
// Integrals whose integrand is a weight times a product of P(ell) values
enum PellKind { K_T1_SQUARE = 0, K_T1_CIRCLE, K_T1_INF, K_T2_A, K_T2_B_SQUARE, K_T2_B_CIRCLE };


template <typename R, int DIM, int KIND>
struct PellProd {
  static constexpr int NCH = 8;  // node chunks of 12 per P(ell)
  static constexpr int NL = (KIND <= K_T1_INF) ? 3 : 1;
  static constexpr int G = NL * NCH;
  static constexpr int PD = 1;
  static constexpr int MINB = 1;
  static constexpr bool CLUSTER16 = false;
  static constexpr int NS = NL;
  __device__ static int slot(int g) { return g / NCH; }
  static constexpr int CH = (DIM == 6) ? 2 : 8;
  struct Rec {
    R ell[3], l2ell[3];
    double wt;
    int valid, los;
  };
  static constexpr int REC = (int)sizeof(Rec);
  const int* job_order = nullptr;
  static constexpr size_t PSMEM = sizeof(R) * HC_COUNT * NNODE + sizeof(CosmoK<R>) + 64;

  const CovJob* jobs;
  const R* hcoef;  // this cosmology's Halofit node table
  CosmoK<R> ck;
  double psn;      // shape-noise power 0.5 sigma^2 / n
  int constant_ps;
  double thetaMax, thetaMaxY;  // survey sides (equal unless rectangular)
  double norm;     // final normalisation of each integral
  double* out;
  int* status;
  // per-job
  R* s_hc;
  double th[6], lmin, lmax;
  int loaded;

  __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) {
    s_hc = (R*)psmem;
    if (!loaded) {
      __syncthreads();
      for (int i = threadIdx.x; i < HC_COUNT * NNODE; i += blockDim.x) s_hc[i] = hcoef[i];
      __syncthreads();
      loaded = 1;
    }
    const CovJob& J = jobs[job];
    for (int i = 0; i < 6; ++i) th[i] = J.th[i];
    lmin = J.lmin;
    lmax = J.lmax;
    if constexpr (KIND == K_T1_SQUARE || KIND == K_T1_CIRCLE) {
      for (int d = 0; d < 6; ++d) {
        xmin[d] = -lmax;
        xmax[d] = 1.02 * lmax;
      }
    } else if constexpr (KIND == K_T1_INF) {
      xmin[0] = lmin, xmin[1] = lmin, xmin[2] = 0;
      xmax[0] = lmax, xmax[1] = lmax, xmax[2] = PI;
    } else if constexpr (KIND == K_T2_B_SQUARE) {
      xmin[0] = -lmax, xmin[1] = -lmax;
      xmax[0] = lmax, xmax[1] = lmax;
    } else {
      xmin[0] = lmin;
      xmax[0] = lmax;
    }
  }

  __device__ bool is_live(const char* r) const { return ((const Rec*)r)->los != 0; }

  __device__ bool setup(int p, const double* x, char* recp) {
    (void)p;
    Rec& r = *(Rec*)recp;
    double ell[3] = {0, 0, 0};
    double wt = 0;
    bool zero = false;
    if constexpr (KIND == K_T1_SQUARE || KIND == K_T1_CIRCLE) {
      double a = x[0], b = x[1], c = x[2], d = x[3], e = x[4], f = x[5];
      ell[0] = sqrt((a - c - e) * (a - c - e) + (b - d - f) * (b - d - f));
      ell[1] = sqrt(c * c + d * d);
      ell[2] = sqrt(e * e + f * f);
      double G;
      if constexpr (KIND == K_T1_SQUARE) {
        G = (double)g_square<R>((R)thetaMax, (R)thetaMaxY, (R)a, (R)b);
        zero = ell[0] <= 0 || ell[1] <= 0 || ell[2] <= 0 || ell[2] > lmax;
      } else {
        G = (double)g_circle<R>((R)thetaMax, (R)sqrt(a * a + b * b));
        zero = ell[0] <= lmin || ell[1] <= lmin || ell[2] <= lmin;
      }
      if (!zero)
        wt = G * uhat(ell[0] * th[0]) * uhat(ell[1] * th[1]) * uhat(ell[2] * th[2]) * uhat(ell[0] * th[3]) *
             uhat(ell[1] * th[4]) * uhat(ell[2] * th[5]);
    } else if constexpr (KIND == K_T1_INF) {
      double l1 = x[0], l2 = x[1], phi = x[2];
      ell[0] = l1;
      ell[1] = l2;
      ell[2] = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi));
      zero = l1 <= lmin || l2 <= lmin || ell[2] <= lmin || ell[2] > lmax;
      if (!zero)
        wt = uhat(l1 * th[0]) * uhat(l2 * th[1]) * uhat(ell[2] * th[2]) * uhat(l1 * th[3]) * uhat(l2 * th[4]) *
             uhat(ell[2] * th[5]) * l1 * l2;
    } else if constexpr (KIND == K_T2_A) {
      ell[0] = x[0];
      zero = ell[0] < lmin;
      if (!zero) wt = ell[0] * uhat(ell[0] * th[0]) * uhat(ell[0] * th[1]);
    } else if constexpr (KIND == K_T2_B_SQUARE) {
      double lx = x[0], ly = x[1];
      ell[0] = sqrt(lx * lx + ly * ly);
      // ell = 0 (the box centre) is the integrand's limit 0; the reference
      // evaluates Pell(0) there, which is NaN
      zero = ell[0] < lmin || ell[0] == 0;
      if (!zero) wt = uhat(ell[0] * th[0]) * uhat(ell[0] * th[1]) * (double)g_square<R>((R)thetaMax, (R)thetaMaxY, (R)lx, (R)ly);
    } else {
      ell[0] = x[0];
      zero = ell[0] < lmin || ell[0] == 0;
      if (!zero) wt = ell[0] * uhat(ell[0] * th[0]) * uhat(ell[0] * th[1]) * (double)g_circle<R>((R)thetaMax, (R)ell[0]);
    }
    r.valid = !zero && wt != 0.0;
    r.los = r.valid && !constant_ps;
    r.wt = wt;
    for (int i = 0; i < NL; ++i) {
      r.ell[i] = (R)ell[i];
      r.l2ell[i] = r.valid ? (R)log2(ell[i]) : (R)0;
    }
    return r.los;
  }

  __device__ void group(const char* recp, int g, double* pv) {
    const Rec& r = *(const Rec*)recp;
    const int i = g / NCH, ch = g % NCH;
    KSum<R> acc;
    const int j0 = ch * (NNODE / NCH);
#pragma unroll 2
    for (int j = j0; j < j0 + NNODE / NCH; ++j) {
      R v = pell_node<R>(s_hc, j, r.ell[i], r.l2ell[i], ck);
      if (v != v) v = (R)0;
      acc.add(v);
    }
    pv[0] = (double)acc.s;
  }

  __device__ void finalize(const char* recp, const double* sum, double* fv) {
    const Rec& r = *(const Rec*)recp;
    if (!r.valid) {
      fv[0] = 0;
      return;
    }
    double v = r.wt;
    for (int i = 0; i < NL; ++i) v *= (r.los ? sum[i] : 0.0) + psn;
    fv[0] = v;
  }

  __device__ void end_job(int job, const double* V, const double* E, long long nev, int st) {
    (void)E;
    (void)nev;
    if (threadIdx.x == 0) {
      out[job] = V[0] * norm;
      if (status) status[job] = st;
    }
  }
};

// ---------------------------------------------------------------------------
// T4: bispectrum-product term, infinite geometry, 5-D in (ln l1, ln l2, ln l5, phi1, phi2)
template <typename R>
struct BkProd {
  static constexpr int G = 16;  // 2 b_kappa x 8 node chunks
  static constexpr int PD = 1;
  static constexpr int MINB = 1;
  static constexpr bool CLUSTER16 = false;
  static constexpr int NS = 2;
  __device__ static int slot(int g) { return g >> 3; }
  static constexpr int CH = 4;
  // FP64 rows NC_* with Tri<double>; FP32 rows NF_* (pair-interleaved, packed
  // node pairs as in k_map3) with TriF
  struct RecD {
    Tri<double> t[2];
    double wt;
    int valid;
  };
  struct RecF {
    TriF t[2];
    double wt;
    int valid;
  };
  typedef typename std::conditional<sizeof(R) == 4, RecF, RecD>::type Rec;
  static constexpr int REC = (int)sizeof(Rec);
  const int* job_order = nullptr;
  static constexpr size_t PSMEM = sizeof(R) * NCP * NNODE + sizeof(CosmoK<R>) + 64;

  const CovJob* jobs;
  const R* ncoef;  // NC_* rows (FP64) or NF_* rows (FP32) of the cosmology
  double wscale;
  CosmoK<R> ck;
  double norm;
  double* out;
  int* status;
  R* s_nc;
  double th[6], lmax;
  int loaded;

  __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) {
    s_nc = (R*)psmem;
    if (!loaded) {
      __syncthreads();
      for (int i = threadIdx.x; i < NCP * NNODE; i += blockDim.x) s_nc[i] = ncoef[i];
      __syncthreads();
      loaded = 1;
    }
    const CovJob& J = jobs[job];
    for (int i = 0; i < 6; ++i) th[i] = J.th[i];
    lmax = J.lmax;
    const double lmin = 1e-5;
    for (int d = 0; d < 3; ++d) {
      xmin[d] = log(lmin);
      xmax[d] = log(lmax);
    }
    xmin[3] = 0, xmin[4] = 0;
    xmax[3] = 2 * PI, xmax[4] = 2 * PI;
  }

  __device__ bool is_live(const char* r) const { return ((const Rec*)r)->valid != 0; }

  __device__ bool setup(int p, const double* x, char* recp) {
    (void)p;
    Rec& r = *(Rec*)recp;
    double l1 = exp(x[0]), l2 = exp(x[1]), l5 = exp(x[2]), c1 = cos(x[3]), c2 = cos(x[4]);
    double l3 = sqrt(l1 * l1 + l2 * l2 + 2 * l1 * l2 * c1);
    double l6 = sqrt(l1 * l1 + l5 * l5 + 2 * l1 * l5 * c2);
    bool zero = l3 > lmax || l6 > lmax || !(l3 > 0) || !(l6 > 0);
    // b_kappa's own cut-offs (bispectrum.cu:295-296,315-318)
    zero = zero || !(l3 > 1e-10) || !(l6 > 1e-10);
    double wt = 0;
    if (!zero) {
      double lp = l1 * l2 * l5;
      wt = uhat(l1 * th[0]) * uhat(l2 * th[1]) * uhat(l3 * th[2]) * uhat(l1 * th[3]) * uhat(l5 * th[4]) *
           uhat(l6 * th[5]) * lp * lp;
    }
    r.valid = !zero && wt != 0.0;
    r.wt = wt;
    if (r.valid) {
      if constexpr (sizeof(R) == 4) {
        Tri<float> t;
        make_tri<float>(l1, l2, l3, t);
        trif_from_tri(t, r.t[0]);
        make_tri<float>(l1, l5, l6, t);
        trif_from_tri(t, r.t[1]);
      } else {
        make_tri<R>(l1, l2, l3, r.t[0]);
        make_tri<R>(l1, l5, l6, r.t[1]);
      }
    }
    return r.valid;
  }

  __device__ void group(const char* recp, int g, double* pv) {
    const Rec& r = *(const Rec*)recp;
    const int i = g >> 3, ch = g & 7;
    const int j0 = ch * 12;
    if constexpr (sizeof(R) == 4) {
      // two nodes per step in packed FP32 pairs with merged reciprocals;
      // Kahan sum per lane. A non-finite sum (a NaN node, which
      // bispectrum.cu:327-331 sets to 0, or a merged product out of the float
      // range) sends the group to the separate-reciprocal form with per-node
      // zeroing.
      float2 sm = make_float2(0.f, 0.f), cmp = make_float2(0.f, 0.f);
      for (int p = j0 / 2; p < (j0 + 12) / 2; ++p) {
        const float2 v = bispec_pair_node<std::remove_cv_t<std::remove_reference_t<decltype(r.t[i])>>, true>(s_nc, p, r.t[i], ck);
        const float2 y = p2sub(v, cmp);
        const float2 t = p2add(sm, y);
        cmp = p2sub(p2sub(t, sm), y);
        sm = t;
      }
      if (!isfinite(sm.x + sm.y)) {
        sm = make_float2(0.f, 0.f), cmp = make_float2(0.f, 0.f);
        for (int p = j0 / 2; p < (j0 + 12) / 2; ++p) {
          float2 v = bispec_pair_node(s_nc, p, r.t[i], ck);
          if (v.x != v.x) v.x = 0.f;
          if (v.y != v.y) v.y = 0.f;
          const float2 y = p2sub(v, cmp);
          const float2 t = p2add(sm, y);
          cmp = p2sub(p2sub(t, sm), y);
          sm = t;
        }
      }
      pv[0] = (double)(sm.x + sm.y);
    } else {
      KSum<R> acc;
#pragma unroll 2
      for (int j = j0; j < j0 + 12; ++j) {
        R v = bispec_node<R>(s_nc, j, r.t[i], ck);
        if (v != v) v = (R)0;
        acc.add(v);
      }
      pv[0] = (double)acc.s;
    }
  }

  __device__ void finalize(const char* recp, const double* sum, double* fv) {
    const Rec& r = *(const Rec*)recp;
    fv[0] = r.valid ? r.wt * (sum[0] * wscale) * (sum[1] * wscale) : 0.0;
  }

  __device__ void end_job(int job, const double* V, const double* E, long long nev, int st) {
    (void)E;
    (void)nev;
    if (threadIdx.x == 0) {
      out[job] = V[0] * norm;
      if (status) status[job] = st;
    }
  }
};


// ---------------------------------------------------------------------------
// host side: permutation tables of the totals, job assembly
struct PermTerm {
  int mult;
  int idx[6];  // into (a0, a1, a2, b0, b1, b2)
};

// T1_total, apertureStatisticsCovariance.cu:272-326
static std::vector<PermTerm> t1_terms(const double* a, const double* b) {
  (void)a;
  if (b[0] == b[1]) {
    if (b[1] == b[2]) return {{6, {0, 1, 2, 3, 3, 3}}};
    return {{2, {0, 1, 2, 3, 3, 5}}, {2, {0, 1, 2, 3, 5, 3}}, {2, {0, 1, 2, 5, 3, 3}}};
  }
  if (b[0] == b[2]) return {{2, {0, 1, 2, 3, 4, 3}}, {2, {0, 1, 2, 3, 3, 4}}, {2, {0, 1, 2, 4, 3, 3}}};
  if (b[1] == b[2]) return {{2, {0, 1, 2, 3, 4, 4}}, {2, {0, 1, 2, 4, 3, 4}}, {2, {0, 1, 2, 4, 4, 3}}};
  return {{1, {0, 1, 2, 3, 4, 5}}, {1, {0, 1, 2, 3, 5, 4}}, {1, {0, 1, 2, 4, 3, 5}},
          {1, {0, 1, 2, 4, 5, 3}}, {1, {0, 1, 2, 5, 3, 4}}, {1, {0, 1, 2, 5, 4, 3}}};
}

// T2_total, apertureStatisticsCovariance.cu:328-538: the first-triplet pattern
// picks the index triples of the first three arguments, the second-triplet
// pattern those of the last three.
static std::vector<PermTerm> t2_terms(const double* a, const double* b) {
  int acase = (a[0] == a[1] && a[1] == a[2]) ? 0 : (a[0] == a[1]) ? 1 : (a[1] == a[2]) ? 2 : (a[0] == a[2]) ? 3 : 4;
  int bcase = (b[0] == b[1] && b[1] == b[2]) ? 0 : (b[0] == b[1]) ? 1 : (b[0] == b[2]) ? 2 : (b[1] == b[2]) ? 3 : 4;
  struct T {
    int m, i0, i1, i2, j0, j1, j2;
  };
  static const std::vector<T> tab[5][5] = {
      // a all equal
      {{{9, 0, 0, 0, 3, 3, 3}},
       {{6, 0, 0, 0, 3, 3, 5}, {3, 0, 0, 0, 5, 3, 3}},
       {{6, 0, 0, 0, 3, 4, 3}, {3, 0, 0, 0, 4, 3, 3}},
       {{6, 0, 0, 0, 4, 3, 4}, {3, 0, 0, 0, 3, 4, 4}},
       {{3, 0, 0, 0, 3, 4, 5}, {3, 0, 0, 0, 4, 3, 5}, {3, 0, 0, 0, 5, 3, 4}}},
      // a0 == a1
      {{{6, 0, 2, 0, 3, 3, 3}, {3, 0, 0, 2, 3, 3, 3}},
       {{2, 0, 0, 2, 3, 3, 5}, {1, 0, 0, 2, 5, 3, 3}, {4, 0, 2, 0, 3, 3, 5}, {2, 0, 2, 0, 5, 3, 3}},
       {{2, 0, 0, 2, 3, 4, 3}, {1, 0, 0, 2, 4, 3, 3}, {4, 0, 2, 0, 3, 4, 3}, {2, 0, 2, 0, 4, 3, 3}},
       {{2, 0, 0, 2, 4, 3, 4}, {1, 0, 0, 2, 3, 4, 4}, {4, 0, 2, 0, 4, 3, 4}, {2, 0, 2, 0, 3, 4, 4}},
       {{1, 0, 0, 2, 3, 4, 5}, {1, 0, 0, 2, 4, 3, 5}, {1, 0, 0, 2, 5, 3, 4},
        {2, 0, 2, 0, 3, 4, 5}, {2, 0, 2, 0, 4, 3, 5}, {2, 0, 2, 0, 5, 3, 4}}},
      // a1 == a2
      {{{6, 0, 1, 1, 3, 3, 3}, {3, 1, 1, 0, 3, 3, 3}},
       {{2, 0, 1, 1, 5, 3, 3}, {1, 1, 1, 0, 5, 3, 3}, {4, 0, 1, 1, 3, 3, 5}, {2, 1, 1, 0, 3, 3, 5}},
       {{4, 0, 1, 1, 3, 4, 3}, {2, 0, 1, 1, 4, 3, 3}, {2, 1, 1, 0, 3, 4, 3}, {1, 1, 1, 0, 4, 3, 3}},
       {{2, 0, 1, 1, 3, 4, 4}, {1, 1, 1, 0, 3, 4, 4}, {4, 0, 1, 1, 4, 3, 4}, {2, 1, 1, 0, 4, 3, 4}},
       {{2, 0, 1, 1, 3, 4, 5}, {2, 0, 1, 1, 4, 3, 5}, {2, 0, 1, 1, 5, 3, 4},
        {1, 1, 1, 0, 3, 4, 5}, {1, 1, 1, 0, 4, 3, 5}, {1, 1, 1, 0, 5, 3, 4}}},
      // a0 == a2
      {{{6, 0, 1, 0, 3, 3, 3}, {3, 1, 0, 0, 3, 3, 3}},
       {{2, 0, 1, 0, 5, 3, 3}, {1, 1, 0, 0, 5, 3, 3}, {4, 0, 1, 0, 3, 3, 5}, {2, 1, 0, 0, 3, 3, 5}},
       {{4, 0, 1, 0, 3, 4, 3}, {2, 0, 1, 0, 4, 3, 3}, {2, 1, 0, 0, 3, 4, 3}, {1, 1, 0, 0, 4, 3, 3}},
       {{2, 0, 1, 0, 3, 4, 4}, {1, 1, 0, 0, 3, 4, 4}, {4, 0, 1, 0, 4, 3, 4}, {2, 1, 0, 0, 4, 3, 4}},
       {{2, 0, 1, 0, 3, 4, 5}, {2, 0, 1, 0, 4, 3, 5}, {2, 0, 1, 0, 5, 3, 4},
        {1, 1, 0, 0, 3, 4, 5}, {1, 1, 0, 0, 4, 3, 5}, {1, 1, 0, 0, 5, 3, 4}}},
      // all different
      {{{3, 0, 1, 2, 3, 3, 3}, {3, 0, 2, 1, 3, 3, 3}, {3, 1, 2, 0, 3, 3, 3}},
       {{2, 0, 1, 2, 3, 3, 5}, {1, 0, 1, 2, 5, 3, 3}, {2, 0, 2, 1, 3, 3, 5},
        {1, 0, 2, 1, 5, 3, 3}, {2, 1, 2, 0, 3, 3, 5}, {1, 1, 2, 0, 5, 3, 3}},
       {{2, 0, 1, 2, 3, 4, 3}, {1, 0, 1, 2, 4, 3, 3}, {2, 0, 2, 1, 3, 4, 3},
        {1, 0, 2, 1, 4, 3, 3}, {2, 1, 2, 0, 3, 4, 3}, {1, 1, 2, 0, 4, 3, 3}},
       {{2, 0, 1, 2, 4, 3, 4}, {1, 0, 1, 2, 3, 4, 4}, {2, 0, 2, 1, 4, 3, 4},
        {1, 0, 2, 1, 3, 4, 4}, {2, 1, 2, 0, 4, 3, 4}, {1, 1, 2, 0, 3, 4, 4}},
       {{1, 0, 1, 2, 3, 4, 5}, {1, 0, 1, 2, 4, 3, 5}, {1, 0, 1, 2, 5, 3, 4},
        {1, 0, 2, 1, 3, 4, 5}, {1, 0, 2, 1, 4, 3, 5}, {1, 0, 2, 1, 5, 3, 4},
        {1, 1, 2, 0, 3, 4, 5}, {1, 1, 2, 0, 4, 3, 5}, {1, 1, 2, 0, 5, 3, 4}}}};
  std::vector<PermTerm> out;
  for (const T& t : tab[acase][bcase]) out.push_back({t.m, {t.i0, t.i1, t.i2, t.j0, t.j1, t.j2}});
  return out;
}

// T4_total, apertureStatisticsCovariance.cu:540-683 (argument patterns as the
// reference evaluates them)
static std::vector<PermTerm> t4_terms(const double* a, const double* b) {
  const double t0 = a[0], t1 = a[1], t2 = a[2], t3 = b[0], t4 = b[1], t5 = b[2];
  if (t0 == t1 && t0 == t2) {
    if (t3 == t4 && t3 == t5) return {{9, {3, 0, 0, 0, 3, 3}}};
    if (t3 == t4) return {{6, {3, 0, 0, 0, 3, 5}}, {3, {5, 0, 0, 0, 3, 3}}};
    return {{3, {3, 0, 0, 0, 4, 5}}, {3, {4, 0, 0, 0, 3, 5}}, {3, {5, 0, 0, 0, 3, 4}}};
  }
  if (t0 == t1) {
    if (t3 == t4 && t3 == t5) return {{6, {3, 0, 2, 0, 3, 3}}, {3, {3, 0, 0, 2, 3, 3}}};
    if (t3 == t4)
      return {{2, {3, 0, 0, 2, 3, 5}}, {4, {3, 0, 2, 0, 3, 5}}, {1, {5, 0, 0, 2, 3, 3}}, {2, {5, 0, 2, 0, 3, 3}}};
    return {{1, {3, 0, 0, 2, 4, 5}}, {2, {3, 0, 2, 0, 4, 5}}, {1, {4, 0, 0, 2, 3, 5}},
            {2, {4, 0, 2, 0, 3, 5}}, {1, {5, 0, 0, 2, 3, 4}}, {2, {5, 0, 2, 0, 3, 4}}};
  }
  if (t3 == t4) {
    if (t3 == t5) return {{3, {3, 0, 1, 2, 3, 3}}, {3, {3, 0, 2, 1, 3, 3}}, {3, {3, 1, 2, 0, 3, 3}}};
    return {{2, {3, 0, 1, 2, 3, 5}}, {2, {3, 0, 2, 1, 3, 5}}, {2, {3, 1, 2, 0, 3, 5}},
            {1, {5, 0, 1, 2, 3, 4}}, {1, {5, 1, 2, 0, 3, 3}}, {1, {5, 0, 2, 1, 3, 3}}};
  }
  if (t4 == t5)
    return {{1, {3, 0, 1, 2, 4, 5}}, {1, {3, 0, 2, 1, 4, 5}}, {1, {3, 1, 2, 0, 4, 4}},
            {2, {4, 0, 1, 2, 3, 4}}, {2, {4, 1, 2, 0, 3, 4}}, {2, {4, 0, 2, 1, 3, 4}}};
  return {{1, {3, 0, 1, 2, 4, 5}}, {1, {3, 0, 2, 1, 4, 5}}, {1, {3, 1, 2, 0, 4, 5}},
          {1, {4, 0, 1, 2, 3, 5}}, {1, {4, 0, 2, 1, 3, 5}}, {1, {4, 1, 2, 0, 3, 5}},
          {1, {5, 0, 1, 2, 3, 4}}, {1, {5, 0, 2, 1, 3, 4}}, {1, {5, 1, 2, 0, 3, 4}}};
}


// T5_total, apertureStatisticsCovariance.cu:685-845. Its second test repeats
// th0 == th1 (:703-705), so whenever th0 == th1 the first triplet is taken as
// (th0, th0, th0); the reference's outputs are defined by that.
static std::vector<PermTerm> t5_terms(const double* a, const double* b) {
  const bool b01 = b[0] == b[1], b12 = b[1] == b[2], b02 = b[0] == b[2];
  if (a[0] == a[1]) {
    if (b01 && b02) return {{9, {0, 0, 0, 3, 3, 3}}};
    if (b01) return {{6, {0, 0, 0, 3, 3, 5}}, {3, {0, 0, 0, 5, 3, 3}}};
    if (b12) return {{3, {0, 0, 0, 3, 4, 4}}, {6, {0, 0, 0, 4, 3, 4}}};
    return {{3, {0, 0, 0, 3, 4, 5}}, {3, {0, 0, 0, 4, 3, 5}}, {3, {0, 0, 0, 5, 3, 4}}};
  }
  if (b01 && b02) return {{3, {0, 1, 2, 3, 3, 3}}, {3, {1, 0, 2, 3, 3, 3}}, {3, {2, 0, 1, 3, 3, 3}}};
  if (b01)
    return {{2, {0, 1, 2, 3, 3, 5}}, {1, {0, 1, 2, 5, 3, 3}}, {2, {1, 0, 2, 3, 4, 5}},
            {1, {1, 0, 2, 5, 3, 3}}, {2, {2, 0, 1, 3, 3, 5}}, {1, {2, 0, 1, 5, 3, 3}}};
  if (b12)
    return {{1, {0, 1, 2, 3, 4, 4}}, {2, {0, 1, 2, 4, 3, 4}}, {1, {1, 0, 2, 3, 4, 4}},
            {2, {1, 0, 2, 4, 3, 4}}, {1, {2, 0, 1, 3, 4, 4}}, {2, {2, 0, 1, 4, 3, 4}}};
  std::vector<PermTerm> out;
  for (const auto& f : {std::array<int, 3>{0, 1, 2}, {1, 0, 2}, {2, 0, 1}})
    for (const auto& g : {std::array<int, 3>{3, 4, 5}, {4, 3, 5}, {5, 3, 4}})
      out.push_back({1, {f[0], f[1], f[2], g[0], g[1], g[2]}});
  return out;
}

// T6_total, apertureStatisticsCovariance.cu:847-1024 (cases A-L)
static std::vector<PermTerm> t6_terms(const double* a, const double* b) {
  const bool b01 = b[0] == b[1], b12 = b[1] == b[2], b02 = b[0] == b[2];
  if (a[0] == a[1] && a[0] == a[2]) {
    if (b01 && b02) return {{3, {0, 0, 0, 3, 3, 3}}, {3, {3, 3, 0, 0, 0, 3}}};
    if (b01) return {{3, {0, 0, 0, 3, 3, 5}}, {1, {3, 3, 0, 0, 0, 5}}, {2, {3, 5, 0, 0, 0, 3}}};
    if (b12) return {{3, {0, 0, 0, 3, 4, 4}}, {2, {3, 4, 0, 0, 0, 4}}, {1, {4, 4, 0, 0, 0, 3}}};
    return {{3, {0, 0, 0, 3, 4, 5}}, {1, {3, 4, 0, 0, 0, 5}}, {1, {3, 5, 0, 0, 0, 4}}, {1, {4, 5, 0, 0, 0, 3}}};
  }
  if (a[0] == a[1]) {
    if (b01 && b02) return {{1, {0, 0, 2, 3, 3, 3}}, {2, {0, 2, 0, 3, 3, 3}}, {3, {3, 3, 0, 0, 2, 3}}};
    if (b01)
      return {{1, {0, 0, 2, 3, 3, 5}}, {2, {0, 2, 0, 3, 3, 5}}, {1, {3, 3, 0, 0, 2, 5}}, {2, {3, 5, 0, 0, 2, 3}}};
    if (b12)
      return {{1, {0, 0, 2, 3, 4, 4}}, {2, {0, 2, 0, 3, 4, 4}}, {2, {3, 4, 0, 0, 2, 4}}, {1, {4, 4, 0, 0, 2, 3}}};
    return {{1, {0, 0, 2, 3, 4, 5}}, {2, {0, 2, 0, 3, 4, 5}}, {1, {3, 4, 0, 0, 2, 5}},
            {1, {3, 5, 0, 0, 2, 4}}, {1, {4, 5, 0, 0, 2, 3}}};
  }
  if (b01 && b02)
    return {{1, {0, 1, 2, 3, 3, 3}}, {1, {0, 2, 1, 3, 3, 3}}, {1, {1, 2, 0, 3, 3, 3}}, {3, {3, 3, 0, 1, 2, 3}}};
  if (b01)
    return {{1, {0, 1, 2, 3, 3, 5}}, {1, {0, 2, 1, 3, 3, 5}}, {1, {1, 2, 0, 3, 3, 5}},
            {1, {3, 3, 0, 1, 2, 5}}, {2, {3, 5, 0, 1, 2, 3}}};
  if (b12)
    return {{1, {0, 1, 2, 3, 4, 4}}, {1, {0, 2, 1, 3, 4, 4}}, {1, {1, 2, 0, 3, 4, 4}},
            {2, {3, 4, 0, 1, 2, 4}}, {1, {4, 4, 0, 1, 2, 3}}};
  return {{1, {0, 1, 2, 3, 4, 5}}, {1, {0, 2, 1, 3, 4, 5}}, {1, {1, 2, 0, 3, 4, 5}},
          {1, {3, 4, 0, 1, 2, 5}}, {1, {3, 5, 0, 1, 2, 4}}, {1, {4, 5, 0, 1, 2, 3}}};
}

// T7_total, apertureStatisticsCovariance.cu:1026-1044: the one ordering
static std::vector<PermTerm> t7_terms(const double*, const double*) { return {{1, {0, 1, 2, 3, 4, 5}}}; }

template <typename R, int DIM, int KIND>
static int run_pell_kind(tp_ctx* ctx, int cosmo, const JobSet& js, double theta_max, double theta_max_y,
                         double norm, double rel_tol, std::vector<double>& res, int& bad) {
  res.assign(js.jobs.size(), 0.0);
  if (js.jobs.empty()) return TP_OK;
  PellProd<R, DIM, KIND> pol;
  memset(&pol, 0, sizeof(pol));
  pol.hcoef = (sizeof(R) == 8 ? (const R*)(const void*)ctx->d_hcoef : (const R*)(const void*)ctx->d_hcoef32) +
              (size_t)cosmo * HC_COUNT * NNODE;
  CosmoK<R> ck;
  cudaError_t e = cudaMemcpyAsync(&ck, (const char*)(sizeof(R) == 8 ? ctx->d_ck64 : ctx->d_ck32) + sizeof(CosmoK<R>) * cosmo,
                                  sizeof(ck), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "cov constants");
  pol.ck = ck;
  pol.psn = 0.5 * ctx->sigma_eps * ctx->sigma_eps / ctx->ngal;
  pol.constant_ps = ctx->constant_ps;
  pol.thetaMax = theta_max;
  pol.thetaMaxY = theta_max_y;
  pol.norm = norm;
  return run_jobs<DIM>(ctx, pol, js.jobs, rel_tol, 0, res, bad);
}

template <typename R>
static int run_t4(tp_ctx* ctx, int cosmo, const JobSet& js, double norm, std::vector<double>& res, int& bad) {
  res.assign(js.jobs.size(), 0.0);
  if (js.jobs.empty()) return TP_OK;
  BkProd<R> pol;
  memset(&pol, 0, sizeof(pol));
  pol.ncoef = (sizeof(R) == 8 ? (const R*)(const void*)ctx->d_ncoef64 : (const R*)(const void*)ctx->d_fcoef32) +
              (size_t)cosmo * NCP * NNODE;
  CosmoK<R> ck;
  double ws = 1.0;
  cudaError_t e = cudaMemcpyAsync(&ck, (const char*)(sizeof(R) == 8 ? ctx->d_ck64 : ctx->d_ck32) + sizeof(CosmoK<R>) * cosmo,
                                  sizeof(ck), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&ws, (sizeof(R) == 8 ? ctx->d_wscale64 : ctx->d_wscale32) + cosmo, sizeof(double),
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "T4 constants");
  pol.ck = ck;
  pol.wscale = ws;
  pol.norm = norm;
  return run_jobs<5>(ctx, pol, js.jobs, 1e-2, 0, res, bad);
}

// Evaluates T_term(th6[i]) for all i (single terms, no permutation sums).
template <typename R>
static int cov_terms(tp_ctx* ctx, int cosmo, int term, int geom, double theta_max, double area,
                     const std::vector<std::array<double, 6>>& th6, std::vector<double>& out, int& bad) {
  const size_t n = th6.size();
  out.assign(n, 0.0);
  const double two_pi = 2 * PI;
  // the rectangle runs the square kinds with its second side
  const bool boxy = geom == TP_GEOM_SQUARE || geom == TP_GEOM_RECTANGLE;
  const double tmy = geom == TP_GEOM_RECTANGLE ? ctx->theta_max_smaller : theta_max;
  if (term == 1) {
    JobSet js;
    std::vector<int> id(n);
    for (size_t i = 0; i < n; ++i) {
      const double* t = th6[i].data();
      double lmax = 10. / std::max(std::min({t[0], t[1], t[2]}), std::min({t[3], t[4], t[5]}));
      id[i] = js.add(t, 6, 0.0, lmax);
    }
    std::vector<double> r;
    int st;
    if (geom == TP_GEOM_INFINITE) {
      if (!(area > 0)) return tp_fail(ctx, TP_ERR_ARG, "T1 (infinite) needs area > 0");
      st = run_pell_kind<R, 3, K_T1_INF>(ctx, cosmo, js, theta_max, tmy, 2 / area / pow(two_pi, 3), 1e-4, r, bad);
    } else if (boxy) {
      st = run_pell_kind<R, 6, K_T1_SQUARE>(ctx, cosmo, js, theta_max, tmy, 1 / pow(two_pi, 6), 1e-2, r, bad);
    } else {
      st = run_pell_kind<R, 6, K_T1_CIRCLE>(ctx, cosmo, js, theta_max, tmy, 1 / pow(two_pi, 6), 1e-2, r, bad);
    }
    if (st) return st;
    for (size_t i = 0; i < n; ++i) out[i] = r[id[i]];
    return TP_OK;
  }
  if (term == 2) {
    if (geom == TP_GEOM_INFINITE) return TP_OK;  // T2 vanishes for an infinite survey
    JobSet ja, jb;
    std::vector<int> i1(n), i2(n), i3(n);
    for (size_t i = 0; i < n; ++i) {
      const double* t = th6[i].data();
      // the 1-D upper bound uses theta1..theta5 and serves both 1-D integrals
      // (apertureStatisticsCovariance.cu:1117-1124)
      double l1 = 10. / std::min({t[0], t[1], t[2], t[3], t[4]});
      double a12[2] = {t[0], t[1]}, a56[2] = {t[4], t[5]}, b34[2] = {t[2], t[3]};
      i1[i] = ja.add(a12, 2, 0.0, l1);
      i2[i] = ja.add(a56, 2, 0.0, l1);
      if (boxy)
        i3[i] = jb.add(b34, 2, 0.0, 10. / std::min(t[2], t[3]));
      else
        i3[i] = jb.add(b34, 2, 0.0, l1);
    }
    std::vector<double> ra, rb;
    int st = run_pell_kind<R, 1, K_T2_A>(ctx, cosmo, ja, theta_max, tmy, 1 / two_pi, 1e-4, ra, bad);
    if (st) return st;
    if (boxy)
      st = run_pell_kind<R, 2, K_T2_B_SQUARE>(ctx, cosmo, jb, theta_max, tmy, 1 / (two_pi * two_pi), 1e-4, rb, bad);
    else
      st = run_pell_kind<R, 1, K_T2_B_CIRCLE>(ctx, cosmo, jb, theta_max, tmy, 1 / two_pi, 1e-4, rb, bad);
    if (st) return st;
    for (size_t i = 0; i < n; ++i) out[i] = ra[i1[i]] * ra[i2[i]] * rb[i3[i]];
    return TP_OK;
  }
  if (term >= 5) {
    if (term != 6 && !(area > 0)) return tp_fail(ctx, TP_ERR_ARG, "T5 and T7 need area > 0");
    int st = halo_terms(ctx, cosmo, term, geom, theta_max, area, th6, sizeof(R) == 4 ? TP_FP32 : TP_FP64, out, bad);
    if (st || term != 6) return st;
    // T6 = (1-D integral over ell_1 of integrand_T2_part1 with (theta1,
    // theta2) on [1e-4, lMax], :1247-1255) x its 7-D halo integral; the
    // integrand's own cut stays at the driver's lMin = 0
    JobSet ja;
    std::vector<int> ia(n);
    for (size_t i = 0; i < n; ++i) {
      const double* t = th6[i].data();
      const double a12[2] = {t[0], t[1]};
      ia[i] = ja.add(a12, 2, HALO_LMIN, halo_lmax(6, t));
    }
    std::vector<double> ra;
    st = run_pell_kind<R, 1, K_T2_A>(ctx, cosmo, ja, theta_max, tmy, 1 / two_pi, 1e-4, ra, bad);
    if (st) return st;
    for (size_t i = 0; i < n; ++i) out[i] *= ra[ia[i]];
    return TP_OK;
  }
  // term 4: infinite geometry with the survey area
  if (!(area > 0)) return tp_fail(ctx, TP_ERR_ARG, "T4 needs area > 0");
  JobSet js;
  std::vector<int> id(n);
  for (size_t i = 0; i < n; ++i) {
    const double* t = th6[i].data();
    double lmax = 10. / std::max(std::min({t[0], t[1], t[2]}), std::min({t[3], t[4], t[5]}));
    id[i] = js.add(t, 6, 1e-5, lmax);
  }
  std::vector<double> r;
  int st = run_t4<R>(ctx, cosmo, js, 1 / area / pow(two_pi, 5), r, bad);
  if (st) return st;
  for (size_t i = 0; i < n; ++i) out[i] = r[id[i]];
  return TP_OK;
}

// ---- P(ell) points ---------------------------------------------------------
template <typename R>
__global__ void k_pell(const double* ell, long n, const R* hcoef, const CosmoK<R>* ckp, double psn, int constant_ps,
                       double* out) {
  long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= n) return;
  double l = ell[w];
  if (constant_ps) {
    if (lane == 0) out[w] = psn;
    return;
  }
  const CosmoK<R> K = *ckp;
  KSum<R> acc;
  R lr = (R)l, l2 = (R)log2(l);
  for (int j = lane; j < NNODE; j += 32) {
    R v = pell_node<R>(hcoef, j, lr, l2, K);
    if (v != v) v = (R)0;
    acc.add(v);
  }
  double s = (double)acc.s;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[w] = s + psn;
}

}  // namespace tp

using namespace tp;

static int check_cov_args(tp_ctx* ctx, int cosmo, int term, int geom, int precision) {
  if (!ctx) return TP_ERR_ARG;
  if (cosmo < 0 || cosmo >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  if (term != 1 && term != 2 && (term < 4 || term > 7)) return tp_fail(ctx, TP_ERR_ARG, "term must be 1, 2, 4, 5, 6 or 7");
  if (geom < TP_GEOM_CIRCLE || geom > TP_GEOM_RECTANGLE) return tp_fail(ctx, TP_ERR_ARG, "unknown geometry");
  // the reference's T4 throws for every geometry but the infinite one (apertureStatisticsCovariance.cu:1183-1195)
  if (term == 4 && geom != TP_GEOM_INFINITE)
    return tp_fail(ctx, TP_ERR_ARG, "T4: only coded for the infinite survey geometry");
  // T5 and T7 likewise (:1227-1230, :1310-1313); T6 for the square and the rectangle (:1235-1238)
  if ((term == 5 || term == 7) && geom != TP_GEOM_INFINITE)
    return tp_fail(ctx, TP_ERR_ARG, "T5/T7: only coded for the infinite survey geometry");
  if (term == 6 && geom == TP_GEOM_CIRCLE)
    return tp_fail(ctx, TP_ERR_ARG, "T6: only coded for square and rectangular survey geometries");
  if (geom == TP_GEOM_RECTANGLE && !(ctx->theta_max_smaller > 0))
    return tp_fail(ctx, TP_ERR_STATE, "rectangular geometry needs tp_set_rectangle_side");
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  return TP_OK;
}

extern "C" int tp_cov_term_batch(tp_ctx* ctx, int cosmo, int term, int geometry, double theta_max, double area,
                                 const double* th6, int n, int precision, double* out, int* status_bad) {
  TpRange nvtx_range("tp_cov_term_batch: covariance terms");
  int st = check_cov_args(ctx, cosmo, term, geometry, precision);
  if (st) return st;
  if (!th6 || !out || n < 0) return TP_ERR_ARG;
  for (int i = 0; i < 6 * n; ++i)
    if (!(th6[i] > 0)) return tp_fail(ctx, TP_ERR_ARG, "aperture radii must be > 0");
  if (term == 6 && geometry == TP_GEOM_INFINITE)
    return tp_fail(ctx, TP_ERR_ARG, "T6: only coded for square and rectangular survey geometries");
  cudaSetDevice(ctx->device);
  std::vector<std::array<double, 6>> v(n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 6; ++k) v[i][k] = th6[6 * i + k];
  std::vector<double> r;
  int bad = 0;
  st = precision == TP_FP64 ? cov_terms<double>(ctx, cosmo, term, geometry, theta_max, area, v, r, bad)
                            : cov_terms<float>(ctx, cosmo, term, geometry, theta_max, area, v, r, bad);
  if (st) return st;
  for (int i = 0; i < n; ++i) out[i] = r[i];
  if (status_bad) *status_bad = bad;
  if (bad) return tp_fail(ctx, TP_ERR_CAPACITY, std::to_string(bad) + " covariance integrals hit a cap");
  return TP_OK;
}

extern "C" int tp_cov_total_batch(tp_ctx* ctx, int cosmo, int term, int geometry, double theta_max, double area,
                                  const double* th123, const double* th456, int n, int precision, double* out,
                                  int* status_bad) {
  TpRange nvtx_range("tp_cov_total_batch: covariance totals");
  int st = check_cov_args(ctx, cosmo, term, geometry, precision);
  if (st) return st;
  if (!th123 || !th456 || !out || n < 0) return TP_ERR_ARG;
  for (int i = 0; i < 3 * n; ++i)
    if (!(th123[i] > 0) || !(th456[i] > 0)) return tp_fail(ctx, TP_ERR_ARG, "aperture radii must be > 0");
  cudaSetDevice(ctx->device);
  std::vector<std::array<double, 6>> all;
  std::vector<std::vector<std::pair<int, int>>> use(n);  // (multiplicity, index into all)
  std::map<std::array<double, 6>, int> seen;
  for (int i = 0; i < n; ++i) {
    const double* a = th123 + 3 * i;
    const double* b = th456 + 3 * i;
    // T2_total and T6_total are 0 for the infinite survey (:330-331, :849-850)
    if ((term == 2 || term == 6) && geometry == TP_GEOM_INFINITE) continue;
    std::vector<PermTerm> terms = term == 1   ? t1_terms(a, b)
                                  : term == 2 ? t2_terms(a, b)
                                  : term == 4 ? t4_terms(a, b)
                                  : term == 5 ? t5_terms(a, b)
                                  : term == 6 ? t6_terms(a, b)
                                              : t7_terms(a, b);
    const double src[6] = {a[0], a[1], a[2], b[0], b[1], b[2]};
    for (const PermTerm& t : terms) {
      std::array<double, 6> th;
      for (int k = 0; k < 6; ++k) th[k] = src[t.idx[k]];
      auto it = seen.find(th);
      int id;
      if (it == seen.end()) {
        id = (int)all.size();
        all.push_back(th);
        seen[th] = id;
      } else {
        id = it->second;
      }
      use[i].push_back({t.mult, id});
    }
  }
  std::vector<double> r;
  int bad = 0;
  st = precision == TP_FP64 ? cov_terms<double>(ctx, cosmo, term, geometry, theta_max, area, all, r, bad)
                            : cov_terms<float>(ctx, cosmo, term, geometry, theta_max, area, all, r, bad);
  if (st) return st;
  for (int i = 0; i < n; ++i) {
    double s = 0;
    for (auto& u : use[i]) s += u.first * r[u.second];
    out[i] = s;
  }
  if (status_bad) *status_bad = bad;
  if (bad) return tp_fail(ctx, TP_ERR_CAPACITY, std::to_string(bad) + " covariance integrals hit a cap");
  return TP_OK;
}

extern "C" int tp_cov_total_terms(int term, int geometry, const double* th123, const double* th456, int* mult,
                                  int* idx, int cap) {
  if (!th123 || !th456 || !mult || !idx || cap < 0) return -1;
  if (term != 1 && term != 2 && (term < 4 || term > 7)) return -1;
  if ((term == 2 || term == 6) && geometry == TP_GEOM_INFINITE) return 0;
  const std::vector<PermTerm> t = term == 1   ? t1_terms(th123, th456)
                                  : term == 2 ? t2_terms(th123, th456)
                                  : term == 4 ? t4_terms(th123, th456)
                                  : term == 5 ? t5_terms(th123, th456)
                                  : term == 6 ? t6_terms(th123, th456)
                                              : t7_terms(th123, th456);
  if ((int)t.size() > cap) return -1;
  for (size_t k = 0; k < t.size(); ++k) {
    mult[k] = t[k].mult;
    for (int j = 0; j < 6; ++j) idx[6 * k + j] = t[k].idx[j];
  }
  return (int)t.size();
}

extern "C" int tp_pell_batch(tp_ctx* ctx, int cosmo, const double* ell, long n, int precision, double* out) {
  if (!ctx || !ell || !out || n < 0) return TP_ERR_ARG;
  if (cosmo < 0 || cosmo >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  for (long i = 0; i < n; ++i)
    if (!(ell[i] > 0)) return tp_fail(ctx, TP_ERR_ARG, "ell must be > 0");
  if (n == 0) return TP_OK;
  cudaSetDevice(ctx->device);
  size_t o_o = (sizeof(double) * n + 255) & ~size_t(255);
  int st = ctx->ensure_io(o_o + sizeof(double) * n + 256);
  if (st) return st;
  char* b = ctx->d_io;
  cudaStream_t s = ctx->stream;
  double psn = 0.5 * ctx->sigma_eps * ctx->sigma_eps / ctx->ngal;
  cudaError_t e = cudaMemcpyAsync(b, ell, sizeof(double) * n, cudaMemcpyHostToDevice, s);
  unsigned grid = (unsigned)((n * 32 + 255) / 256);
  if (e == cudaSuccess) {
    if (precision == TP_FP64)
      k_pell<double><<<grid, 256, 0, s>>>((double*)b, n, ctx->d_hcoef + (size_t)cosmo * HC_COUNT * NNODE,
                                          (const CosmoK<double>*)ctx->d_ck64 + cosmo, psn, ctx->constant_ps,
                                          (double*)(b + o_o));
    else
      k_pell<float><<<grid, 256, 0, s>>>((double*)b, n, ctx->d_hcoef32 + (size_t)cosmo * HC_COUNT * NNODE,
                                         (const CosmoK<float>*)ctx->d_ck32 + cosmo, psn, ctx->constant_ps,
                                         (double*)(b + o_o));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, b + o_o, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return tp_cuda(ctx, e, "pell");
}
