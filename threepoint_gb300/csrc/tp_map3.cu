// <Map^3> integrand and its batched adaptive integration.
//
// Reference: integrand_Map3_kernel (cuda_version/apertureStatistics.cu:138-153),
// MapMapMap (:201-230), bkappa / GQ96_of_bdelta / integrand_bkappa
// (cuda_version/bispectrum.cu:293-333), uHat (apertureStatistics.cu:18-22).
//
// One integral = one (cosmology, theta-triplet) job. Point record: the
// triangle (ell1, ell2, ell3), its shape factors and the outer factor
// l1 l2 uHat(l1 t1) uHat(l2 t2) uHat(l3 t3); the 96 line-of-sight nodes of
// b_kappa are split into G groups of 96/G nodes, one (point, group) item per
// thread. The node table of the job's cosmology (NC_COUNT x 96) is staged in
// shared memory with a bulk async copy when the CTA switches cosmology.
#include <cuda_runtime.h>

#include <algorithm>

#include <type_traits>

#include "tp_bispec.cuh"
#include "tp_cubature.cuh"
#include "tp_internal.cuh"
#include "tp_kernels.cuh"

// Launch shape of the FP32 kernel: resident CTAs per SM requested from the
// register allocator, and how many line-of-sight nodes one thread evaluates
// per loop iteration (build-time tuning knobs, see threepoint_gb300/build.py).
#ifndef TP_MAP3_MINB
#define TP_MAP3_MINB 3
#endif
#ifndef TP_MAP3_UNROLL
#define TP_MAP3_UNROLL 1
#endif
#ifndef TP_MAP3_DUP_IN_LOOP
#define TP_MAP3_DUP_IN_LOOP 1
#endif
// 1: the FP32 linear-P(k) table is read from global memory through L1 instead
// of being staged in shared memory (16 KB less per CTA, so four 256-thread
// CTAs fit an SM's shared memory)
#ifndef TP_MAP3_PLT_GLOBAL
#define TP_MAP3_PLT_GLOBAL 0
#endif
#define TP_PRAGMA(x) _Pragma(#x)
#define TP_UNROLL(n) TP_PRAGMA(unroll n)

namespace tp {

template <typename R>
struct Map3Policy {
  static constexpr int G = 8;              // node groups per point
  static constexpr int NPG = NNODE / G;    // nodes per group
  static constexpr int CH = 8;             // regions per evaluation chunk
  // Point records are read by consecutive threads for consecutive points, so
  // the FP32 record has an odd number of 32-bit words (17): conflict-free
  // shared-memory banks. FP32 keeps the filter product as its log2.
  struct RecF {
    TriF tri;
    float lo;  // log2(l1 l2 uHat uHat uHat)
    int live;
  };
  struct RecD {
    Tri<double> tri;
    double outer;  // l1 l2 uHat uHat uHat
    int live;
  };
  typedef typename std::conditional<sizeof(R) == 4, RecF, RecD>::type Rec;
  const int* job_order;
  static constexpr int REC = (int)sizeof(Rec);
  static constexpr int PD = 1;
  static constexpr int NS = 1;
  __device__ static int slot(int) { return 0; }
  static constexpr size_t PLT_BYTES = (sizeof(R) == 4 && !TP_MAP3_PLT_GLOBAL) ? sizeof(float4) * PLT_N : 0;
  static constexpr size_t PSMEM = sizeof(R) * NCP * NNODE + sizeof(CosmoK<R>) + sizeof(BulkBar) + 128 + PLT_BYTES;

  // inputs
  const int* job_cosmo;
  const double* job_theta;
  const R* node_coef;        // [n_cosmo][NNODE][NCP]: NC_* rows (FP64) or NF_* rows (FP32), weights / wscale
  const double* wscale;      // [n_cosmo]
  const CosmoK<R>* ck;       // [n_cosmo]
  double lmin, lmax, phimin, phimax;
  // outputs
  double* out;
  double* err;
  int64_t* neval;
  int64_t* nlive;
  int* status;
  unsigned* diag;
  // per-CTA state
  R* s_nc;
  CosmoK<R>* s_ck;
  int cur_cosmo;
  double th[3];
  float thf[3];
  double scale;

  __device__ BulkBar* bar(char* psmem) {
    return (BulkBar*)(psmem + sizeof(R) * NCP * NNODE + ((sizeof(CosmoK<R>) + 15) & ~size_t(15)));
  }
  __device__ unsigned long long* live_counter(char* psmem) {
    return (unsigned long long*)((char*)bar(psmem) + ((sizeof(BulkBar) + 15) & ~size_t(15)));
  }
  __device__ float4* plt_smem(char* psmem) { return (float4*)((char*)live_counter(psmem) + 16); }
  unsigned long long* s_live;

  __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) {
    s_nc = (R*)psmem;
    s_ck = (CosmoK<R>*)(psmem + sizeof(R) * NCP * NNODE);
    const int c = job_cosmo[job];
    if (c != cur_cosmo) {
      __syncthreads();
      const R* src = node_coef + (size_t)c * NCP * NNODE;
      constexpr int nbytes = (int)(sizeof(R) * NCP * NNODE);
      static_assert(nbytes % 16 == 0, "bulk copy size must be a multiple of 16 bytes");
      if (threadIdx.x == 0) {
        // the node table (10-20 KB) is staged by one bulk async copy
        if (!bulk_copy_g2s(bar(psmem), s_nc, src, nbytes)) {
          for (int i = 0; i < NCP * NNODE; ++i) s_nc[i] = src[i];
        }
        *s_ck = ck[c];
      }
      __syncthreads();
      if constexpr (sizeof(R) == 4 && !TP_MAP3_PLT_GLOBAL) {
        // the FP32 linear-P(k) table follows the node table into shared memory
        const float4* gp = reinterpret_cast<const float4*>(s_ck->plt);
        if (gp) {
          float4* sp = plt_smem(psmem);
          for (int i = threadIdx.x; i < PLT_N; i += blockDim.x) sp[i] = gp[i];
          __syncthreads();
          if (threadIdx.x == 0) s_ck->plt = reinterpret_cast<const float*>(sp);
        }
      }
      __syncthreads();
      cur_cosmo = c;
    }
    th[0] = job_theta[3 * job];
    th[1] = job_theta[3 * job + 1];
    th[2] = job_theta[3 * job + 2];
    thf[0] = (float)th[0];
    thf[1] = (float)th[1];
    thf[2] = (float)th[2];
    double tmin = fmin(th[0], fmin(th[1], th[2]));
    double lm = lmax > 0 ? lmax : 10. / tmin;
    xmin[0] = lmin;
    xmin[1] = lmin;
    xmin[2] = phimin;
    xmax[0] = lm;
    xmax[1] = lm;
    xmax[2] = phimax;
    scale = wscale[c];
    s_live = live_counter(psmem);
    if (threadIdx.x == 0) *s_live = 0ull;
    __syncthreads();
  }

  // returns whether the point needs its line-of-sight sum
  __device__ bool setup(int p, const double* x, char* recp) {
    (void)p;
    Rec& r = *(Rec*)recp;
    bool live;
    if constexpr (sizeof(R) == 4) {
      // FP32 path: the whole point setup in FP32 (FP64 issues ~60x slower)
      typedef Mth<float> M;
      float l1 = (float)x[0], l2 = (float)x[1];
      float sh, ch;
      __sincosf(0.5f * (float)x[2], &sh, &ch);
      float cphi = 1.f - 2.f * sh * sh;
      float d = l1 - l2;
      float l3 = sqrtf(d * d + 4.f * l1 * l2 * ch * ch);
      // log2 of the filter product l1 l2 uHat uHat uHat, so that its dynamic
      // range is that of FP64 (values far below the float range still steer
      // the adaptive refinement as they do in the FP64 path)
      const float LOG2E = 1.4426950408889634f;
      float t1 = 0.5f * (l1 * thf[0]) * (l1 * thf[0]);
      float t2 = 0.5f * (l2 * thf[1]) * (l2 * thf[1]);
      float t3 = 0.5f * (l3 * thf[2]) * (l3 * thf[2]);
      live = l1 > 1.0e-10f && l2 > 1.0e-10f && l3 > 1.0e-10f && t1 > 0.f && t2 > 0.f && t3 > 0.f;
      float L = M::lg2(l1 * l2) + M::lg2(t1) + M::lg2(t2) + M::lg2(t3) - LOG2E * (t1 + t2 + t3);
      live = live && L > -1070.f;
      r.lo = L;
      if (live) {
        Tri<float> t;
        make_tri_phi_f(l1, l2, cphi, l3, t);
        trif_from_tri(t, r.tri);
      }
    } else {
      double l1 = x[0], l2 = x[1], phi = x[2];
      double s = l1 * l1 + l2 * l2 + 2 * l1 * l2 * cos(phi);
      double l3 = s > 0 ? sqrt(s) : 0.0;
      double outer = l1 * l2 * uhat(l1 * th[0]) * uhat(l2 * th[1]) * uhat(l3 * th[2]);
      live = !(l1 == 0 || l2 == 0 || l3 == 0) && l1 > 1.0e-10 && l2 > 1.0e-10 && l3 > 1.0e-10 && outer != 0.0;
      r.outer = outer;
      if (live) make_tri<R>(l1, l2, l3, r.tri);
    }
    r.live = live;
    if (live && nlive) atomicAdd(s_live, 1ull);
    return live;
  }

  // line-of-sight partial sum over node group g (only called for live points)
  __device__ void group(const char* recp, int g, double* pv) {
    const Rec& r = *(const Rec*)recp;
    const CosmoK<R>& K = *s_ck;  // fields read from shared memory where used
    const int j0 = g * NPG;
    if constexpr (sizeof(R) == 4) {
      // two nodes per step in packed FP32 pairs; Kahan sum per lane
#if TP_MAP3_DUP_IN_LOOP
      const TriF& T2 = r.tri;  // pairs formed where used
#else
      TriF2 T2;  // pairs held in registers across the node loop
      trif2_from(r.tri, T2, K.lgp_lo, K.lgp_hi);
#endif
      // Nodes with merged reciprocals. A NaN node (bispectrum.cu:327-331 sets
      // it to 0), an infinite one or a merged product out of the float range
      // makes the Kahan sum non-finite: then, rarely, the group is summed
      // again with separate reciprocals and the per-node zeroing, which gives
      // the same result as zeroing on every node.
      float2 s = make_float2(0.f, 0.f), cmp = make_float2(0.f, 0.f);
      TP_UNROLL(TP_MAP3_UNROLL)
      for (int p = j0 / 2; p < (j0 + NPG) / 2; ++p) {
        const float2 v = bispec_pair_node<std::remove_cv_t<std::remove_reference_t<decltype(T2)>>, true>(s_nc, p, T2, K);
        const float2 y = p2sub(v, cmp);
        const float2 t = p2add(s, y);
        cmp = p2sub(p2sub(t, s), y);
        s = t;
      }
      if (!isfinite(s.x + s.y)) {
        s = make_float2(0.f, 0.f), cmp = make_float2(0.f, 0.f);
        for (int p = j0 / 2; p < (j0 + NPG) / 2; ++p) {
          float2 v = bispec_pair_node(s_nc, p, T2, K);
          if (v.x != v.x) v.x = 0.f;
          if (v.y != v.y) v.y = 0.f;
          const float2 y = p2sub(v, cmp);
          const float2 t = p2add(s, y);
          cmp = p2sub(p2sub(t, s), y);
          s = t;
        }
      }
      pv[0] = (double)(s.x + s.y);  // lanes added in FP32: one conversion, no FP64 add per item
    } else {
      KSum<R> acc;
      TP_UNROLL(TP_MAP3_UNROLL)
      for (int j = j0; j < j0 + NPG; ++j) {
        R v = bispec_node<R>(s_nc, j, r.tri, K);
        if (v != v) v = (R)0;  // NaN in bispec -> 0 (bispectrum.cu:327-331)
        acc.add(v);
      }
      pv[0] = (double)acc.s;
    }
  }

  __device__ bool is_live(const char* recp) const { return ((const Rec*)recp)->live != 0; }

  __device__ void finalize(const char* recp, const double* sum, double* fv) {
    const Rec& r = *(const Rec*)recp;
    if (!r.live) {
      fv[0] = 0.0;
      return;
    }
    double outer;
    if constexpr (sizeof(R) == 4)
      outer = (r.lo > -120.f) ? (double)Mth<float>::ex2(r.lo) : exp2((double)r.lo);
    else
      outer = r.outer;
    fv[0] = outer * scale * sum[0];
  }

  // called by rank 0 of a cluster (or the CTA) after the last sweep; the
  // live-point counters of the other ranks are read through distributed
  // shared memory (they are reset only at their next job, after a barrier
  // rank 0 has not yet reached)
  __device__ void end_job(int job, const double* V, const double* E, long long nev, int st) {
    if (threadIdx.x == 0) {
      const double norm = 1. / 8 / PI / PI / PI;
      out[job] = V[0] * norm;
      if (err) err[job] = E[0] * norm;
      if (neval) neval[job] = nev;
      if (nlive) {
        unsigned long long live = *s_live;
        cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        for (unsigned r = 1; r < cl.num_blocks(); ++r) live += *cl.map_shared_rank(s_live, r);
        nlive[job] = (int64_t)live;
      }
      if (status) status[job] = st;
    }
  }
};

// CS > 1: one cluster of CS CTAs per integral (the cooperative form of
// adaptive_body), for batches with fewer integrals than CTA slots
template <typename R, int NT, int CS>
__global__ void __launch_bounds__(NT, sizeof(R) == 4 ? TP_MAP3_MINB : 1) k_map3(Map3Policy<R> pol_in, int njobs, int* job_counter, EngineCfg cfg,
                                             char* scratch, size_t slot_bytes) {
  Map3Policy<R> pol = pol_in;
  pol.cur_cosmo = -1;
  extern __shared__ __align__(16) char smem_[];
  BulkBar* b = pol.bar(smem_);
  if (threadIdx.x == 0) bulkbar_init(b);
  __syncthreads();
  adaptive_body<3, 1, NT, Map3Policy<R>, CS>(pol, njobs, job_counter, cfg, scratch, slot_bytes);
  if (threadIdx.x == 0 && b->timeouts && pol.diag) atomicAdd(pol.diag, b->timeouts);
}

template <typename R>
size_t map3_smem_bytes() {
  typedef Map3Policy<R> P;
  constexpr int NP = GMRule<3>::NP;
  size_t b = (P::PSMEM + 15) & ~size_t(15);
  b += ((size_t)P::CH * NP * P::REC + 15) & ~size_t(15);
  b += sizeof(double) * (size_t)P::G * P::CH * NP;
  b += sizeof(double) * (size_t)P::CH * NP;
  b += sizeof(EngineShared<1>) + 16;
  return b;
}

// ---------------------------------------------------------------------------
// Point evaluation of b_kappa (no cubature): one warp per point, 3 nodes per
// lane, shuffle reduction.
template <typename R>
__global__ void k_bkappa_points(const int* cosmo_idx, const double* ell, long n, const R* node_coef,
                                const double* wscale, const CosmoK<R>* ck, double* out) {
  long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= n) return;
  int c = cosmo_idx ? cosmo_idx[w] : 0;
  double l1 = ell[3 * w], l2 = ell[3 * w + 1], l3 = ell[3 * w + 2];
  if (l1 == 0 || l2 == 0 || l3 == 0 || !(l1 > 1e-10 && l2 > 1e-10 && l3 > 1e-10)) {
    if (lane == 0) out[w] = 0.0;
    return;
  }
  Tri<R> T;
  make_tri<R>(l1, l2, l3, T);
  const R* nc = node_coef + (size_t)c * NCP * NNODE;
  const CosmoK<R> K = ck[c];
  KSum<R> acc;
  if constexpr (sizeof(R) == 4) {
    TriF F;
    trif_from_tri(T, F);
    for (int j = lane; j < NNODE; j += 32) {
      float v = bispec_node_fast(nc, j, F, K);
      if (v != v) v = 0.f;
      acc.add(v);
    }
  } else {
    for (int j = lane; j < NNODE; j += 32) {
      R v = bispec_node<R>(nc, j, T, K);
      if (v != v) v = (R)0;
      acc.add(v);
    }
  }
  double s = (double)acc.s;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[w] = s * wscale[c];
}

// Per-node terms of b_kappa at given triangles (no cubature), with the
// functions of the integration kernels: term[i * NNODE + j] is node j's
// line-of-sight term of triangle i (Gauss weight, 27/8 Om^3 (H0/c)^5 and
// (g(1+z))^3 / f_K / E(z) included, NaN -> 0 as integrand_bkappa does,
// bispectrum.cu:311-333), so that the terms of a triangle sum to b_kappa;
// bis (optional) is B(ell / f_K(z_j), z_j) itself (bispec, :221-291).
// FP64: one thread per (triangle, node), bispec_eval on the NC_* rows. FP32:
// one thread per (triangle, node pair), the packed pair evaluation of k_map3
// (merged reciprocals, and the separate-reciprocal form with the per-node
// zeroing when a merged product leaves the float range).
template <typename R>
__global__ void k_bkappa_nodes(int c, const double* ell, long n, const R* node_coef, const double* wscale,
                               const CosmoK<R>* ck, double* term, double* bis) {
  constexpr int PER = sizeof(R) == 4 ? NNODE / 2 : NNODE;
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * PER) return;
  const long i = t / PER;
  const int u = (int)(t % PER);
  const double l1 = ell[3 * i], l2 = ell[3 * i + 1], l3 = ell[3 * i + 2];
  const int j0 = sizeof(R) == 4 ? 2 * u : u, nj = sizeof(R) == 4 ? 2 : 1;
  if (!(l1 > 1e-10 && l2 > 1e-10 && l3 > 1e-10)) {
    for (int q = 0; q < nj; ++q) {
      term[i * NNODE + j0 + q] = 0.0;
      if (bis) bis[i * NNODE + j0 + q] = 0.0;
    }
    return;
  }
  const R* nc = node_coef + (size_t)c * NCP * NNODE;
  const CosmoK<R> K = ck[c];
  Tri<R> T;
  make_tri<R>(l1, l2, l3, T);
  if constexpr (sizeof(R) == 4) {
    TriF F;
    trif_from_tri(T, F);
    const float2* cp = reinterpret_cast<const float2*>(nc) + (size_t)u * NCP;
    float2 B = bispec_pair<TriF, true>(cp, F, K);
    float2 v = p2mul(cp[NF_W], B);
    if (!isfinite(v.x + v.y)) {
      B = bispec_pair<TriF, false>(cp, F, K);
      v = p2mul(cp[NF_W], B);
      if (v.x != v.x) v.x = 0.f;
      if (v.y != v.y) v.y = 0.f;
    }
    term[i * NNODE + j0] = (double)v.x * wscale[c];
    term[i * NNODE + j0 + 1] = (double)v.y * wscale[c];
    if (bis) {
      bis[i * NNODE + j0] = (double)B.x;
      bis[i * NNODE + j0 + 1] = (double)B.y;
    }
  } else {
    const R* row = nc + (size_t)u * NCP;
    const R B = bispec_eval<R>(row, 1, row[NC_S], row[NC_L2S], row[NC_HF], row[NC_L2HF], T, K);
    R v = row[NC_W] * B;
    if (v != v) v = (R)0;
    term[i * NNODE + u] = (double)v * wscale[c];
    if (bis) bis[i * NNODE + u] = (double)B;
  }
}

cudaError_t launch_bkappa_nodes(int precision, int cosmo, const double* ell, long n, const void* ncoef,
                                const double* wscale, const void* ck, double* term, double* bis, cudaStream_t st) {
  const long per = precision == TP_FP64 ? NNODE : NNODE / 2;
  const int bs = 192;
  const unsigned grid = (unsigned)((n * per + bs - 1) / bs);
  if (precision == TP_FP64)
    k_bkappa_nodes<double><<<grid, bs, 0, st>>>(cosmo, ell, n, (const double*)ncoef, wscale,
                                                 (const CosmoK<double>*)ck, term, bis);
  else
    k_bkappa_nodes<float><<<grid, bs, 0, st>>>(cosmo, ell, n, (const float*)ncoef, wscale,
                                                (const CosmoK<float>*)ck, term, bis);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
constexpr int MAP3_NT = 256;

constexpr int MAP3_CLUSTER = 8;

static cudaLaunchConfig_t map3_launch_config(int grid, size_t smem, cudaStream_t st, int cluster,
                                             cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(grid);
  lc.blockDim = dim3(MAP3_NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.attrs = attr;
  lc.numAttrs = cluster > 1 ? 1 : 0;
  return lc;
}

// grid of CTAs (a multiple of *cluster), one CTA per integral, or one
// MAP3_CLUSTER-CTA cluster per integral (*cluster = MAP3_CLUSTER) when
// allow_cluster is 1 and the batch has no more integrals than CTA slots, or
// allow_cluster is 2;
// *scratch = bytes of the region stores (one per CTA or per cluster)
template <typename R>
static cudaError_t plan_map3_t(int njobs, int cap, int max_ctas, int allow_cluster, int* grid, int* cluster,
                               size_t* smem, size_t* scratch) {
  *smem = map3_smem_bytes<R>();
  *cluster = 1;
  cudaError_t e =
      cudaFuncSetAttribute(k_map3<R, MAP3_NT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_map3<R, MAP3_NT, 1>, MAP3_NT, *smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int g = sms * per_sm;
  if (max_ctas > 0 && g > max_ctas) g = max_ctas;
  if ((allow_cluster == 2 || (allow_cluster == 1 && njobs <= g)) && (max_ctas <= 0 || max_ctas >= MAP3_CLUSTER)) {
    int nclusters = 0;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t lc = map3_launch_config(MAP3_CLUSTER, *smem, 0, MAP3_CLUSTER, attr);
    e = cudaFuncSetAttribute(k_map3<R, MAP3_NT, MAP3_CLUSTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)*smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveClusters(&nclusters, (const void*)k_map3<R, MAP3_NT, MAP3_CLUSTER>, &lc);
    cudaGetLastError();
    if (e == cudaSuccess && nclusters >= 1) {
      if (max_ctas > 0) nclusters = std::min(nclusters, max_ctas / MAP3_CLUSTER);
      nclusters = std::min(nclusters, njobs);
      *cluster = MAP3_CLUSTER;
      *grid = nclusters * MAP3_CLUSTER;
      *scratch = (size_t)nclusters * Slot<3, 1>::bytes(cap);
      return cudaSuccess;
    }
  }
  if (g > njobs) g = njobs;
  if (g < 1) g = 1;
  *grid = g;
  *scratch = (size_t)g * Slot<3, 1>::bytes(cap);
  return cudaSuccess;
}

cudaError_t map3_f32_resident_smem(size_t* bytes) {
  const size_t smem = map3_smem_bytes<float>();
  cudaError_t e =
      cudaFuncSetAttribute(k_map3<float, MAP3_NT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, per_sm = 0, reserved = 0;
  cudaGetDevice(&dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_map3<float, MAP3_NT, 1>, MAP3_NT, smem);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  *bytes = (size_t)per_sm * (smem + (size_t)reserved);
  return e;
}

cudaError_t plan_map3(int precision, int njobs, int cap, int max_ctas, int allow_cluster, int* grid, int* cluster,
                      size_t* smem, size_t* scratch) {
  return precision == TP_FP64
             ? plan_map3_t<double>(njobs, cap, max_ctas, allow_cluster, grid, cluster, smem, scratch)
             : plan_map3_t<float>(njobs, cap, max_ctas, allow_cluster, grid, cluster, smem, scratch);
}

template <typename R>
static cudaError_t launch_map3_t(const Map3Launch& L, int grid, size_t smem, char* scratch, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(L.job_counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  Map3Policy<R> pol;
  pol.job_cosmo = L.job_cosmo;
  pol.job_theta = L.job_theta;
  pol.node_coef = (const R*)(sizeof(R) == 8 ? (const void*)L.ncoef64 : (const void*)L.fcoef32);
  pol.wscale = sizeof(R) == 8 ? L.wscale64 : L.wscale32;
  pol.ck = (const CosmoK<R>*)(sizeof(R) == 8 ? L.ck64 : L.ck32);
  pol.lmin = L.lmin;
  pol.lmax = L.lmax;
  pol.phimin = L.phimin;
  pol.phimax = L.phimax;
  pol.out = L.out;
  pol.err = L.err;
  pol.neval = L.neval;
  pol.nlive = L.nlive;
  pol.status = L.status;
  pol.diag = L.diag;
  pol.job_order = L.job_order;
  EngineCfg cfg{0.0, L.rel_tol, TP_NORM_L1, L.cap, L.max_sweeps};
  size_t slot = Slot<3, 1>::bytes(L.cap);
  if (L.cluster == MAP3_CLUSTER) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t lc = map3_launch_config(grid, smem, st, MAP3_CLUSTER, attr);
    return cudaLaunchKernelEx(&lc, k_map3<R, MAP3_NT, MAP3_CLUSTER>, pol, L.njobs, L.job_counter, cfg, scratch, slot);
  }
  k_map3<R, MAP3_NT, 1><<<grid, MAP3_NT, smem, st>>>(pol, L.njobs, L.job_counter, cfg, scratch, slot);
  return cudaGetLastError();
}

cudaError_t launch_map3(const Map3Launch& L, int grid, size_t smem, char* scratch, cudaStream_t st) {
  return L.precision == TP_FP64 ? launch_map3_t<double>(L, grid, smem, scratch, st)
                                : launch_map3_t<float>(L, grid, smem, scratch, st);
}

cudaError_t launch_bkappa_points(int precision, const int* cosmo_idx, const double* ell, long n, const void* ncoef,
                                 const double* wscale, const void* ck, double* out, cudaStream_t st) {
  long threads = n * 32;
  int bs = 256;
  unsigned grid = (unsigned)((threads + bs - 1) / bs);
  if (precision == TP_FP64)
    k_bkappa_points<double><<<grid, bs, 0, st>>>(cosmo_idx, ell, n, (const double*)ncoef, wscale,
                                                  (const CosmoK<double>*)ck, out);
  else
    k_bkappa_points<float><<<grid, bs, 0, st>>>(cosmo_idx, ell, n, (const float*)ncoef, wscale,
                                                 (const CosmoK<float>*)ck, out);
  return cudaGetLastError();
}

}  // namespace tp
