// Natural components Gamma^0..Gamma^3 of the shear three-point correlation
// function: 3-D adaptive cubature over (z, phi, psi) of the Ogata Hankel sum
// of the BiHalofit convergence bispectrum at redshift z.
//
// Reference: gamma0..gamma3 (cuda_version/gamma.cu:98-148), the integrands
// full_integrand_gamma0/1 and one_integrand_gamma0 (:419-482), the triangle
// geometry interior_angle, A, alpha, betabar, prefactor (:484-529), the Ogata
// nodes of compute_weights_bessel (:13-68) and the orthocentre-to-centroid
// rotation (:72-96; CONVERT_TO_CENTROID, gamma.cuh:25).
//
// One job = (triangle, component). A point record holds the z-only BiHalofit
// coefficients of its redshift, the unit triangle shape (cos psi, sin psi,
// ...) and per cyclic term j the scale A_j and complex weight C_j; a
// (point, group) item evaluates 4 Ogata nodes x 3 terms = 12 bispectra.
#include <cuda_runtime.h>

#include <type_traits>

// resident CTAs per SM requested for the FP32 Gamma kernel (2: <= 128
// registers per thread; 1: no register cap, one CTA per SM)
#ifndef TP_GAMMA_MINB
#define TP_GAMMA_MINB 2
#endif

#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "tp_bispec.cuh"
#include "tp_capi_internal.h"
#include "tp_cubature.cuh"
#include "tp_internal.cuh"
#include "tp_kernels.cuh"

namespace tp {

constexpr int PREC_K = 33;       // int(3.31/0.1) Ogata nodes (index 0 unused), gamma.cuh:29-30
constexpr double PREC_H = 0.1;

struct OgataTab {
  double psi[2][PREC_K], prod[2][PREC_K], l2psi[2][PREC_K];  // [0]: J6 (Gamma0), [1]: J2 (Gamma1)
};
__constant__ OgataTab c_og;

// zeros of J_nu by Newton iteration from McMahon's expansion (s >= 1); s = 0 -> 0
static double bessel_zero(int nu, int s) {
  if (s == 0) return 0.0;
  double mu = 4.0 * nu * nu;
  double b = (s + 0.5 * nu - 0.25) * PI;
  double x = b - (mu - 1) / (8 * b) - 4 * (mu - 1) * (7 * mu - 31) / (3 * pow(8 * b, 3));
  if (s == 1) x = nu + 1.8557571 * cbrt((double)nu) + 1.033150 / cbrt((double)nu);
  for (int it = 0; it < 100; ++it) {
    double J = std::cyl_bessel_j((double)nu, x);
    double dJ = 0.5 * (std::cyl_bessel_j((double)nu - 1, x) - std::cyl_bessel_j((double)nu + 1, x));
    double dx = J / dJ;
    x -= dx;
    if (fabs(dx) < 1e-15 * x) break;
  }
  return x;
}

static void ogata_host(OgataTab& o) {
  for (int pass = 0; pass < 2; ++pass) {
    int nu = pass == 0 ? 6 : 2;
    for (int i = 0; i < PREC_K; ++i) {
      double zr = bessel_zero(nu, i), pz = zr / PI;
      double t = pz * PREC_H;
      double psi = PI * (t * tanh(PI * sinh(t) / 2)) / PREC_H;
      double psip = (sinh(PI * sinh(t)) + PI * t * cosh(t)) / (cosh(PI * sinh(t)) + 1);
      double Jn1 = i == 0 ? 0.0 : std::cyl_bessel_j((double)nu + 1, zr);
      double w = 2 / (PI * zr * Jn1 * Jn1);
      o.psi[pass][i] = psi;
      o.prod[pass][i] = i == 0 ? 0.0 : w * psi * psi * psi * std::cyl_bessel_j((double)nu, psi) * psip;
      o.l2psi[pass][i] = i == 0 ? 0.0 : log2(psi);
    }
  }
}

cudaError_t gamma_upload_constants() {
  static OgataTab o;
  static bool built = false;
  if (!built) {
    ogata_host(o);
    built = true;
  }
  return cudaMemcpyToSymbol(c_og, &o, sizeof(o));
}

// geometry (gamma.cu:491-529), double precision
__host__ __device__ inline double interior_angle(double an1, double an2, double opp) {
  return acos((an1 * an1 + an2 * an2 - opp * opp) / (2.0 * an1 * an2));
}
__host__ __device__ inline double height_of_triangle(double x1, double x2, double x3) {
  return 0.5 * sqrt(2 * x1 * x1 + 2 * x2 * x2 - x3 * x3);
}
__host__ __device__ inline double one_rotation_angle_otc(double x1, double x2, double x3) {
  double psi3 = interior_angle(x1, x2, x3);
  double h3 = height_of_triangle(x1, x2, x3);
  double d = x2 * x2 - x1 * x1;
  double s = x1 * x2 * sin(psi3);
  double c2 = (d * d - 4 * s * s) / ((2 * h3 * x3) * (2 * h3 * x3));
  double s2 = d * x1 * x2 * sin(psi3) / ((h3 * x3) * (h3 * x3));
  return atan2(s2, c2) / 2;
}

struct GammaJobs {
  const double* x;  // [n_tri][3]
  const int* comp;  // [n_jobs]
  const int* tri;   // [n_jobs]
};

template <typename R>
struct GammaPolicy {
  static constexpr int G = 8;     // groups of 4 Ogata nodes
  static constexpr int KPG = 4;
  static constexpr int CH = 4;    // regions per chunk (records are large)
  // FP64: the per-point NC_* coefficients (bispec_eval); FP32: the folded
  // NF_* row (bispec_fast_row), an odd number of words (57) per record
  struct RecD {
    double zc[NC_COUNT];
    Tri<double> tri;  // unit-scale triangle (cos psi, sin psi, ell3/psi_k)
    double invA[3], l2A[3];
    double cre[3], cim[3];
    double bmin;
    int live;
  };
  struct RecF {
    float nf[NCP];
    TriF tri;
    float invA[3], l2A[3];
    float cre[3], cim[3];
    float bmin;
    int live;
  };
  typedef typename std::conditional<sizeof(R) == 4, RecF, RecD>::type Rec;
  static constexpr int REC = (int)sizeof(Rec);
  const int* job_order = nullptr;
  static constexpr int PD = 2;
  static constexpr int NS = 1;
  __device__ static int slot(int) { return 0; }
  static constexpr size_t PSMEM = sizeof(CosmoK<R>) + 64;

  GammaJobs J;
  const TablesDev* tab;
  const CosmoDev* cosm;
  const CosmoK<R>* ck;
  int cosmo;
  double* out;  // [n_tri][4][2]
  int* status;  // [n_tri]
  // per-job state
  CosmoK<R>* s_ck;
  int which;                      // 0: Gamma0 integrand, 1: Gamma1 integrand
  double x1, x2, x3;              // sides passed to the integrand (permuted for Gamma2/3)
  double vp[3], ph0[3];           // Gamma0: varpsi_j, constant phase of term j
  double p1, p2, p3;              // Gamma1: interior angles
  double zmax;

  __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) {
    s_ck = (CosmoK<R>*)psmem;
    if (threadIdx.x == 0) *s_ck = ck[cosmo];
    const int t = J.tri[job], c = J.comp[job];
    double a = J.x[3 * t], b = J.x[3 * t + 1], d = J.x[3 * t + 2];
    which = c == 0 ? 0 : 1;
    if (c <= 1) {
      x1 = a, x2 = b, x3 = d;
    } else if (c == 2) {
      x1 = b, x2 = d, x3 = a;  // gamma2 = gamma1(x2, x3, x1)
    } else {
      x1 = d, x2 = a, x3 = b;  // gamma3 = gamma1(x3, x1, x2)
    }
    const double xs[3][3] = {{x1, x2, x3}, {x2, x3, x1}, {x3, x1, x2}};
    for (int j = 0; j < 3; ++j) {
      vp[j] = interior_angle(xs[j][0], xs[j][1], xs[j][2]);
      ph0[j] = interior_angle(xs[j][1], xs[j][2], xs[j][0]) - interior_angle(xs[j][0], xs[j][2], xs[j][1]);
    }
    p1 = interior_angle(x2, x3, x1);
    p2 = interior_angle(x3, x1, x2);
    p3 = interior_angle(x1, x2, x3);
    zmax = cosm[cosmo].zmax;
    xmin[0] = 0;
    xmin[1] = 0;
    xmin[2] = 0;
    xmax[0] = zmax;
    xmax[1] = 2 * PI;
    xmax[2] = PI / 2;
    __syncthreads();
  }

  __device__ bool is_live(const char* recp) const { return ((const Rec*)recp)->live != 0; }

  __device__ bool setup(int p, const double* x, char* recp) {
    (void)p;
    Rec& r = *(Rec*)recp;
    const double z = x[0], phi = x[1], psi = x[2];
    if constexpr (sizeof(R) == 4) {
      float zc[NC_COUNT];
      r.live = zcoefs<float>(tab[cosmo], cosm[cosmo], z, zc);
      if (r.live) nf_from_nc(zc, r.nf);
    } else {
      r.live = zcoefs<R>(tab[cosmo], cosm[cosmo], z, r.zc);
    }
    if (!r.live) return false;
    // the geometry is evaluated in double: a few dozen operations per point
    // against 96 bispectra
    double cp = cos(psi), sp = sin(psi), s2p = sin(2 * psi), c2p = cos(2 * psi);
    double cph = cos(phi), sph = sin(phi);
    double bb = 0.5 * atan2(c2p * sph, cph + s2p);  // betabar, gamma.cu:524-529
    double b3s = cp * cp + sp * sp + 2 * cp * sp * cph;
    double b3 = b3s <= 0 ? 0.0 : sqrt(b3s);
    r.bmin = (R)fmin(cp, fmin(sp, b3));
    if (!(b3 > 0 && cp > 0 && sp > 0)) {
      r.live = 0;
      return false;
    }
    if constexpr (sizeof(R) == 4) {
      Tri<float> t;
      make_tri_phi_f((float)cp, (float)sp, (float)cph, (float)b3, t);
      trif_from_tri(t, r.tri);
    } else {
      make_tri<R>(cp, sp, b3, r.tri);
    }
    if (which == 0) {
      const double xs[3][2] = {{x1, x2}, {x2, x3}, {x3, x1}};
      for (int j = 0; j < 3; ++j) {
        double a = xs[j][0], b = xs[j][1];
        double ang = phi + vp[j];
        double A = sqrt((cp * b) * (cp * b) + (sp * a) * (sp * a) + s2p * a * b * cos(ang));
        double al = atan2((cp * b - sp * a) * sin(ang / 2), (cp * b + sp * a) * cos(ang / 2));
        double phase = ph0[j] - 6 * al + 2 * bb;
        double mag = s2p * PI / (A * A * A * A);
        r.invA[j] = (R)(1.0 / A);
        r.l2A[j] = (R)log2(A);
        r.cre[j] = (R)(mag * cos(phase));
        r.cim[j] = (R)(mag * sin(phase));
      }
    } else {
      // term order as full_integrand_gamma1: j=0 -> A1, 1 -> A2, 2 -> A3
      const double ab[3][2] = {{x2, x3}, {x3, x1}, {x1, x2}};
      const double vps[3] = {p1, p2, p3};
      double ph[3];
      double alv[3], Av[3];
      for (int j = 0; j < 3; ++j) {
        double a = ab[j][0], b = ab[j][1];
        double ang = phi + vps[j];
        Av[j] = sqrt((cp * b) * (cp * b) + (sp * a) * (sp * a) + s2p * a * b * cos(ang));
        alv[j] = atan2((cp * b - sp * a) * sin(ang / 2), (cp * b + sp * a) * cos(ang / 2));
      }
      ph[0] = p3 - p2 - 2 * (bb + alv[0]);
      ph[1] = p3 - p1 - 2 * p2 + 2 * (bb + phi - alv[1]);
      ph[2] = p1 - p2 + 2 * p3 + 2 * (bb - phi - alv[2]);
      for (int j = 0; j < 3; ++j) {
        double mag = s2p * PI / (Av[j] * Av[j] * Av[j] * Av[j]);
        r.invA[j] = (R)(1.0 / Av[j]);
        r.l2A[j] = (R)log2(Av[j]);
        r.cre[j] = (R)(mag * cos(ph[j]));
        r.cim[j] = (R)(mag * sin(ph[j]));
      }
    }
    return true;
  }

  __device__ void group(const char* recp, int g, double* pv) {
    const Rec& r = *(const Rec*)recp;
    const CosmoK<R> K = *s_ck;
    const int og = which;
    KSum<R> are, aim;
    if constexpr (sizeof(R) == 4) {
      const float* c = r.nf;
      const float W = c[NF_W];
      for (int kk = 0; kk < KPG; ++kk) {
        const int k = 1 + g * KPG + kk;
        const float psik = (float)c_og.psi[og][k], l2psik = (float)c_og.l2psi[og][k], prodk = (float)c_og.prod[og][k];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float sc = psik * r.invA[j];
          if (r.bmin * sc <= 1.0e-10f) continue;  // integrand_bkappa: ell <= 1e-10 -> 0
          const TriF T = trif_scaled(r.tri, sc, l2psik - r.l2A[j]);
          float v = W * bispec_fast_row(c, T, K);
          if (v != v) v = 0.f;  // NaN -> 0 (bispectrum.cu:327-331)
          v *= prodk;
          are.add(r.cre[j] * v);
          aim.add(r.cim[j] * v);
        }
      }
    } else {
      const R* zc = r.zc;
      const R s = zc[NC_S], l2s = zc[NC_L2S], hf = zc[NC_HF], l2hf = zc[NC_L2HF], W = zc[NC_W];
      for (int kk = 0; kk < KPG; ++kk) {
        const int k = 1 + g * KPG + kk;
        const R psik = (R)c_og.psi[og][k], l2psik = (R)c_og.l2psi[og][k], prodk = (R)c_og.prod[og][k];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          R sc = psik * r.invA[j];
          if (r.bmin * sc <= (R)1.0e-10) continue;  // integrand_bkappa: ell <= 1e-10 -> 0
          R l2sc = l2psik - r.l2A[j];
          R B = bispec_eval<R>(zc, 1, s * sc, l2s + l2sc, hf * sc, l2hf + l2sc, r.tri, K);
          R v = W * B;
          if (v != v) v = (R)0;  // NaN -> 0 (bispectrum.cu:327-331)
          v *= prodk;
          are.add(r.cre[j] * v);
          aim.add(r.cim[j] * v);
        }
      }
    }
    pv[0] = (double)are.s;
    pv[1] = (double)aim.s;
  }

  __device__ void finalize(const char* recp, const double* sum, double* fv) {
    const Rec& r = *(const Rec*)recp;
    fv[0] = r.live ? sum[0] : 0.0;
    fv[1] = r.live ? sum[1] : 0.0;
  }

  __device__ void end_job(int job, const double* V, const double* E, long long nev, int st) {
    (void)E;
    (void)nev;
    if (threadIdx.x != 0) return;
    const int t = J.tri[job], c = J.comp[job];
    double re = V[0], im = V[1];
    // orthocentre -> centroid (gamma.cu:83-91); Gamma1..3 conjugate phi1
    double a1 = one_rotation_angle_otc(x2, x3, x1), a2 = one_rotation_angle_otc(x3, x1, x2),
           a3 = one_rotation_angle_otc(x1, x2, x3);
    if (c != 0) a1 = -a1;
    double ang = -2. * (a1 + a2 + a3);
    double cr = re * cos(ang) - im * sin(ang), ci = re * sin(ang) + im * cos(ang);
    double om = cosm[cosmo].om;
    double f = 27. / 8. * om * om * om * pow(100. / 299792., 5.0) / 3. / (2 * pow(2 * PI, 3.0));
    out[8 * t + 2 * c] = cr * f;
    out[8 * t + 2 * c + 1] = ci * f;
    if (status && st) atomicOr(&status[t], st);
  }
};

// CS > 1: one cluster of CS CTAs per integral (cooperative adaptive_body)
template <typename R, int NT, int CS>
__global__ void __launch_bounds__(NT, sizeof(R) == 4 ? TP_GAMMA_MINB : 1) k_gamma(GammaPolicy<R> pol_in, int njobs, int* job_counter, EngineCfg cfg,
                                              char* scratch, size_t slot_bytes) {
  GammaPolicy<R> pol = pol_in;
  adaptive_body<3, 2, NT, GammaPolicy<R>, CS>(pol, njobs, job_counter, cfg, scratch, slot_bytes);
}

// The Gamma integrand at caller-given points (no cubature): the policy's
// point set-up and its node groups, summed over the groups, one thread per
// point; dynamic shared memory GammaPolicy<R>::PSMEM.
template <typename R>
__global__ void k_gamma_points(GammaPolicy<R> pol, const double* pts, int n, double* out) {
  extern __shared__ __align__(16) char psmem_[];
  double xmin[3], xmax[3];
  pol.begin_job(0, psmem_, xmin, xmax);
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    alignas(16) char rec[GammaPolicy<R>::REC];
    double sum[2] = {0.0, 0.0}, fv[2];
    if (pol.setup(p, pts + 3 * p, rec)) {
      for (int g = 0; g < GammaPolicy<R>::G; ++g) {
        double pv[2];
        pol.group(rec, g, pv);
        sum[0] += pv[0];
        sum[1] += pv[1];
      }
    }
    pol.finalize(rec, sum, fv);
    out[2 * p] = fv[0];
    out[2 * p + 1] = fv[1];
  }
}

template <typename R>
static size_t gamma_smem_bytes() {
  return engine_smem_bytes<3, 2, GammaPolicy<R>>();
}

constexpr int GAMMA_NT = 256;
constexpr int GAMMA_CLUSTER = 8;

// max_stores: region stores the launch may use (one per CTA, or per cluster),
// 0 = no limit beyond ctx->max_ctas. A batch with no more integrals than CTA
// slots runs one GAMMA_CLUSTER-CTA cluster per integral.
template <typename R>
static int run_gamma(tp_ctx* ctx, int cosmo, const double* d_x, const int* d_comp, const int* d_tri, int njobs,
                     double rel_tol, double* d_out, int* d_status, int cap, int max_stores) {
  size_t smem = gamma_smem_bytes<R>();
  cudaError_t e =
      cudaFuncSetAttribute(k_gamma<R, GAMMA_NT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "gamma attribute");
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gamma<R, GAMMA_NT, 1>, GAMMA_NT, smem);
  if (e != cudaSuccess || per_sm < 1) return tp_cuda(ctx, e == cudaSuccess ? cudaErrorInvalidConfiguration : e, "gamma occupancy");
  int slots = sms * per_sm;
  if (ctx->max_ctas > 0 && slots > ctx->max_ctas) slots = ctx->max_ctas;
  int cluster = 1, units = slots;
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = GAMMA_CLUSTER;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.blockDim = dim3(GAMMA_NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = ctx->stream;
  lc.attrs = attr;
  lc.numAttrs = 1;
  if (njobs <= slots && slots >= GAMMA_CLUSTER) {
    int ncl = 0;
    lc.gridDim = dim3(GAMMA_CLUSTER);
    e = cudaFuncSetAttribute(k_gamma<R, GAMMA_NT, GAMMA_CLUSTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveClusters(&ncl, (const void*)k_gamma<R, GAMMA_NT, GAMMA_CLUSTER>, &lc);
    cudaGetLastError();
    ncl = std::min(ncl, slots / GAMMA_CLUSTER);
    if (e == cudaSuccess && ncl >= 1) {
      cluster = GAMMA_CLUSTER;
      units = ncl;
    }
  }
  if (max_stores > 0 && units > max_stores) units = max_stores;
  if (units > njobs) units = njobs;
  size_t slot = Slot<3, 2>::bytes(cap);
  int st = ctx->ensure_scratch((size_t)units * slot);
  if (st) return st;
  GammaPolicy<R> pol;
  pol.J.x = d_x;
  pol.J.comp = d_comp;
  pol.J.tri = d_tri;
  pol.tab = ctx->d_tab;
  pol.cosm = ctx->d_cos;
  pol.ck = (const CosmoK<R>*)(sizeof(R) == 8 ? ctx->d_ck64 : ctx->d_ck32);
  pol.cosmo = cosmo;
  pol.out = d_out;
  pol.status = d_status;
  EngineCfg cfg{0.0, rel_tol, TP_NORM_L1, cap, 2000};
  e = cudaMemsetAsync(ctx->d_counter, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) {
    if (cluster > 1) {
      lc.gridDim = dim3(units * GAMMA_CLUSTER);
      e = cudaLaunchKernelEx(&lc, k_gamma<R, GAMMA_NT, GAMMA_CLUSTER>, pol, njobs, ctx->d_counter, cfg,
                             ctx->d_scratch, slot);
    } else {
      k_gamma<R, GAMMA_NT, 1><<<units, GAMMA_NT, smem, ctx->stream>>>(pol, njobs, ctx->d_counter, cfg, ctx->d_scratch,
                                                                    slot);
      e = cudaGetLastError();
    }
  }
  return tp_cuda(ctx, e, "gamma launch");
}

}  // namespace tp

using namespace tp;

extern "C" int tp_ogata_weights(double* out) {
  if (!out) return TP_ERR_ARG;
  OgataTab o;
  ogata_host(o);
  for (int k = 0; k < PREC_K; ++k) {
    out[k] = o.psi[0][k];
    out[PREC_K + k] = k == 0 ? NAN : o.prod[0][k];
    out[2 * PREC_K + k] = o.psi[1][k];
    out[3 * PREC_K + k] = k == 0 ? NAN : o.prod[1][k];
  }
  return TP_OK;
}

extern "C" int tp_gamma_integrand_points(tp_ctx* ctx, int cosmo_index, const double* x, int which, const double* pts,
                                         int n, int precision, double* out) {
  TpRange nvtx_range("tp_gamma_integrand_points");
  if (!ctx || !x || !pts || !out || n < 0 || (which != 0 && which != 1)) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (cosmo_index < 0 || cosmo_index >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  if (!(x[0] > 0 && x[1] > 0 && x[2] > 0)) return tp_fail(ctx, TP_ERR_ARG, "triangle sides must be > 0");
  if (n == 0) return TP_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e = gamma_upload_constants();
  if (e != cudaSuccess) return tp_cuda(ctx, e, "ogata constants");
  const int jc[2] = {which, 0};  // job 0: component `which` of triangle 0
  const size_t o_c = 256, o_p = 512, o_o = o_p + ((sizeof(double) * 3 * n + 255) & ~size_t(255));
  int st = ctx->ensure_io(o_o + sizeof(double) * 2 * n + 256);
  if (st) return st;
  char* b = ctx->d_io;
  cudaStream_t s = ctx->stream;
  e = cudaMemcpyAsync(b, x, sizeof(double) * 3, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_c, jc, sizeof(jc), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_p, pts, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "gamma points upload");
  const int nt = 128;
  if (precision == TP_FP64) {
    GammaPolicy<double> pol;
    pol.J.x = (const double*)b;
    pol.J.comp = (const int*)(b + o_c);
    pol.J.tri = (const int*)(b + o_c) + 1;
    pol.tab = ctx->d_tab;
    pol.cosm = ctx->d_cos;
    pol.ck = (const CosmoK<double>*)ctx->d_ck64;
    pol.cosmo = cosmo_index;
    pol.out = nullptr;
    pol.status = nullptr;
    k_gamma_points<double><<<1, nt, GammaPolicy<double>::PSMEM, s>>>(pol, (const double*)(b + o_p), n,
                                                                      (double*)(b + o_o));
  } else {
    GammaPolicy<float> pol;
    pol.J.x = (const double*)b;
    pol.J.comp = (const int*)(b + o_c);
    pol.J.tri = (const int*)(b + o_c) + 1;
    pol.tab = ctx->d_tab;
    pol.cosm = ctx->d_cos;
    pol.ck = (const CosmoK<float>*)ctx->d_ck32;
    pol.cosmo = cosmo_index;
    pol.out = nullptr;
    pol.status = nullptr;
    k_gamma_points<float><<<1, nt, GammaPolicy<float>::PSMEM, s>>>(pol, (const double*)(b + o_p), n,
                                                                    (double*)(b + o_o));
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, b + o_o, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return tp_cuda(ctx, e, "gamma points");
}

// One pass of the Gamma integrals of n triangles (components of comp_mask)
// at region cap `cap` on at most max_ctas CTAs (0: all resident); out is
// [n][4] complex as 8 doubles, status_out[n] the OR of the triangle's
// components' engine status (bit 1: region cap reached).
static int gamma_pass(tp_ctx* ctx, int cosmo_index, const double* x, int n, int comp_mask, double rel_tol,
                      int precision, int cap, int max_ctas, double* out, int* status_out) {
  std::vector<int> comp, tri;
  for (int t = 0; t < n; ++t)
    for (int c = 0; c < 4; ++c)
      if (comp_mask & (1 << c)) {
        comp.push_back(c);
        tri.push_back(t);
      }
  const int nj = (int)comp.size();
  size_t o_x = 0, o_c = (sizeof(double) * 3 * n + 255) & ~size_t(255);
  size_t o_t = o_c + ((sizeof(int) * nj + 255) & ~size_t(255));
  size_t o_o = o_t + ((sizeof(int) * nj + 255) & ~size_t(255));
  size_t o_s = o_o + ((sizeof(double) * 8 * n + 255) & ~size_t(255));
  int st = ctx->ensure_io(o_s + sizeof(int) * n + 256);
  if (st) return st;
  char* b = ctx->d_io;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(b + o_x, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_c, comp.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + o_t, tri.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b + o_o, 0, sizeof(double) * 8 * n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b + o_s, 0, sizeof(int) * n, s);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "gamma upload");
  st = precision == TP_FP64
           ? run_gamma<double>(ctx, cosmo_index, (double*)(b + o_x), (int*)(b + o_c), (int*)(b + o_t), nj, rel_tol,
                               (double*)(b + o_o), (int*)(b + o_s), cap, max_ctas)
           : run_gamma<float>(ctx, cosmo_index, (double*)(b + o_x), (int*)(b + o_c), (int*)(b + o_t), nj, rel_tol,
                              (double*)(b + o_o), (int*)(b + o_s), cap, max_ctas);
  if (st) return st;
  e = cudaMemcpyAsync(out, b + o_o, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(status_out, b + o_s, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return tp_cuda(ctx, e, "gamma");
}

// The reference integrates Gamma with an unbounded hcubature_v (maxEval = 0,
// gamma.cu:110). Triangles whose integrals reach the context's region cap are
// integrated again, from the start, with a cap 16 times larger on as many
// CTAs as fit GAMMA_ESCALATE_BYTES of region stores, up to the context's
// escalation cap (at most GAMMA_CAP_MAX regions per integral); the adaptive
// sequence is deterministic, so the larger cap continues exactly where the
// smaller one stopped. Only what still reaches the last cap is reported.
constexpr int GAMMA_CAP_MAX = 1 << 24;
constexpr size_t GAMMA_ESCALATE_BYTES = size_t(32) << 30;

extern "C" int tp_gamma_batch(tp_ctx* ctx, int cosmo_index, const double* x, int n, int comp_mask, double rel_tol,
                              int precision, double* out, int* status_out) {
  TpRange nvtx_range("tp_gamma_batch: Gamma");
  if (!ctx || !x || !out || n < 0 || (comp_mask & ~0xF) || comp_mask == 0) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (!(rel_tol > 0)) return TP_ERR_ARG;
  if (cosmo_index < 0 || cosmo_index >= ctx->n_cosmo) return tp_fail(ctx, TP_ERR_STATE, "no such cosmology");
  for (int i = 0; i < 3 * n; ++i)
    if (!(x[i] > 0)) return tp_fail(ctx, TP_ERR_ARG, "triangle sides must be > 0");
  for (int t = 0; t < n; ++t) {
    double a = x[3 * t], b = x[3 * t + 1], c = x[3 * t + 2];
    if (a > b + c || b > a + c || c > a + b) return tp_fail(ctx, TP_ERR_ARG, "sides violate the triangle inequality");
  }
  if (n == 0) return TP_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e = gamma_upload_constants();
  if (e != cudaSuccess) return tp_cuda(ctx, e, "ogata constants");
  std::vector<int> hst(n);
  int st = gamma_pass(ctx, cosmo_index, x, n, comp_mask, rel_tol, precision, ctx->region_cap, ctx->max_ctas, out,
                      hst.data());
  if (st) return st;
  for (int cap = ctx->region_cap; cap < std::min(GAMMA_CAP_MAX, ctx->escalate_cap);) {
    std::vector<int> again;
    for (int t = 0; t < n; ++t)
      if (hst[t] & 1) again.push_back(t);
    if (again.empty()) break;
    cap = (int)std::min<long>((long)cap * 16, std::min(GAMMA_CAP_MAX, ctx->escalate_cap));
    const int nj = (int)again.size() * __builtin_popcount((unsigned)comp_mask);
    int ctas = (int)std::max<size_t>(1, GAMMA_ESCALATE_BYTES / Slot<3, 2>::bytes(cap));
    if (ctx->max_ctas > 0) ctas = std::min(ctas, ctx->max_ctas);
    ctas = std::min(ctas, nj);
    std::vector<double> xs(3 * again.size()), os(8 * again.size());
    std::vector<int> ss(again.size());
    for (size_t k = 0; k < again.size(); ++k)
      for (int q = 0; q < 3; ++q) xs[3 * k + q] = x[3 * again[k] + q];
    st = gamma_pass(ctx, cosmo_index, xs.data(), (int)again.size(), comp_mask, rel_tol, precision, cap, ctas,
                    os.data(), ss.data());
    if (st) return st;
    for (size_t k = 0; k < again.size(); ++k) {
      for (int q = 0; q < 8; ++q) out[8 * again[k] + q] = os[8 * k + q];
      hst[again[k]] = ss[k];
    }
  }
  // region stores grown by the escalation are released again
  if (ctx->scratch_bytes > (size_t(4) << 30)) {
    cudaFree(ctx->d_scratch);
    ctx->d_scratch = nullptr;
    ctx->scratch_bytes = 0;
  }
  int bad = 0;
  for (int t = 0; t < n; ++t) {
    if (status_out) status_out[t] = hst[t];
    bad += hst[t] != 0;
  }
  if (bad) return tp_fail(ctx, TP_ERR_CAPACITY, std::to_string(bad) + " Gamma integrals hit a region or sweep cap");
  return TP_OK;
}
