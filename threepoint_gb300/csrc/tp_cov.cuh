// Shared pieces of the covariance integrals (tp_cov.cu: T1, T2, T4;
// tp_halo.cu: the halo-model terms T5, T6, T7): the P_kappa node term, the
// survey windows, the integral job list and the persistent engine launch.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "tp_bispec.cuh"
#include "tp_capi_internal.h"
#include "tp_cubature.cuh"
#include "tp_internal.cuh"

namespace tp {

// P_kappa line-of-sight term of node j at ell (bispectrum.cu:531-600,951-991):
// W_j * T17(k) * P_nl(k, z_j), k = ell / f_K(z_j).
template <typename R>
__device__ __forceinline__ R pell_node(const R* __restrict__ hc, int j, R ell, R l2ell, const CosmoK<R>& K) {
  typedef Mth<R> M;
  const R W = hc[HC_W * NNODE + j];
  if (W == (R)0) return (R)0;
  const R k = ell * hc[HC_INVFK * NNODE + j];
  const R l2k = l2ell + hc[HC_L2INVFK * NNODE + j];
  const R P = plin<R>(K, k * K.h, l2k + K.l2h);
  const R k3 = k * k * k;
  const R pl = P * hc[HC_D1SQ * NNODE + j] * k3 * (R)(1.0 / (2 * PI * PI));
  const R l2y = l2k + hc[HC_L2RS * NNODE + j];
  const R y = k * hc[HC_RS * NNODE + j];
  const R ysq = y * y;
  R ph = hc[HC_A * NNODE + j] * M::ex2((R)3 * hc[HC_F1 * NNODE + j] * l2y) *
         M::rcp((R)1 + hc[HC_B * NNODE + j] * M::ex2(hc[HC_F2 * NNODE + j] * l2y) +
                M::ex2(((R)3 - hc[HC_GAM * NNODE + j]) * (hc[HC_L2F3C * NNODE + j] + l2y)));
  ph = ph * ysq * M::rcp(ysq + hc[HC_XNU * NNODE + j]);
  const R pq = pl * M::ex2(hc[HC_BETA * NNODE + j] * M::lg2((R)1 + pl)) * M::rcp((R)1 + pl * hc[HC_ALPHA * NNODE + j]) *
               M::ex2(-(y * (R)0.25 + ysq * (R)0.125) * (R)1.4426950408889634);
  const R pnl = (R)(2 * PI * PI) * (pq + ph) * M::rcp(k3);
  // T17 correction (bispectrum.cu:971-979)
  const R a1 = (R)1.3063, a2 = (R)1.1475, a3 = (R)0.62793, c1 = (R)9.5171e-4, c2 = (R)5.1543e-3;
  const R corr = M::ex2(a1 * M::lg2((R)1 + c1 * M::ex2(-a1 * l2k)) - a3 * M::lg2((R)1 + c2 * M::ex2(-a2 * l2k)));
  return W * corr * pnl;
}

// windows of the survey geometries (apertureStatisticsCovariance.cu:117-153)
// G_square is the rectangle with two equal sides; G_rectangle (:154-172) has
// side thetaMax along lx and thetaMax_smaller along ly
template <typename R>
__device__ inline R g_square(R thetaMax, R thetaMaxY, R lx, R ly) {
  R t1 = (R)0.5 * lx * thetaMax, t2 = (R)0.5 * ly * thetaMaxY;
  R j1 = fabs(t1) <= (R)1e-6 ? (R)1 : sin(t1) / t1;
  R j2 = fabs(t2) <= (R)1e-6 ? (R)1 : sin(t2) / t2;
  return j1 * j1 * j2 * j2;
}
template <typename R>
__device__ inline R g_circle(R thetaMax, R ell) {
  R t = thetaMax * ell;
  R r = j1(t);
  return r * r * (R)4 / (t * t);
}

struct CovJob {
  double th[6];
  double lmin, lmax;
};

// distinct integrals of one kind
struct JobSet {
  std::vector<CovJob> jobs;
  std::map<std::vector<double>, int> index;
  int add(const double* th, int nth, double lmin, double lmax) {
    std::vector<double> key(th, th + nth);
    key.push_back(lmin);
    key.push_back(lmax);
    auto it = index.find(key);
    if (it != index.end()) return it->second;
    CovJob j;
    memset(&j, 0, sizeof(j));
    for (int i = 0; i < nth; ++i) j.th[i] = th[i];
    j.lmin = lmin;
    j.lmax = lmax;
    int id = (int)jobs.size();
    jobs.push_back(j);
    index[key] = id;
    return id;
  }
};

// Runs the adaptive engine over njobs integrals of policy P, each to relative
// tolerance rel_tol in the L1 norm, on a persistent grid: one CTA per
// integral (CS = 1) or one cluster of CS CTAs per integral (CS > 1, the
// cooperative form of adaptive_body, for integrands whose points are costly
// enough that one integral should spread over several SMs).
// P::MINB: CTAs per SM the register allocation must allow
template <int DIM, class P, int NT, int CS>
__global__ void __launch_bounds__(NT, P::MINB) k_cov(P pol_in, int njobs, int* job_counter, EngineCfg cfg,
                                                     char* scratch, size_t slot_bytes) {
  P pol = pol_in;
  pol.loaded = 0;
  adaptive_body<DIM, 1, NT, P, CS>(pol, njobs, job_counter, cfg, scratch, slot_bytes);
}

template <int DIM, class P, int CS>
inline int run_engine_cs(tp_ctx* ctx, const P& pol, int njobs, double rel_tol, int cap) {
  constexpr int NT = 256;
  if (njobs == 0) return TP_OK;
  auto kern = k_cov<DIM, P, NT, CS>;
  size_t smem = engine_smem_bytes<DIM, 1, P>();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // clusters of more than 8 CTAs are a non-portable size (allowed on GB300)
  if (e == cudaSuccess && CS > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "cov attribute");
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  lc.blockDim = dim3(NT);
  lc.dynamicSmemBytes = smem;
  lc.stream = ctx->stream;
  lc.attrs = attr;
  lc.numAttrs = CS > 1 ? 1 : 0;
  int units = 0;  // integrals in flight: CTAs (CS = 1) or clusters
  if constexpr (CS == 1) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
    if (e != cudaSuccess || per_sm < 1) return tp_cuda(ctx, e ? e : cudaErrorInvalidConfiguration, "cov occupancy");
    units = sms * per_sm;
  } else {
    lc.gridDim = dim3(CS);
    e = cudaOccupancyMaxActiveClusters(&units, (const void*)kern, &lc);
    if (e != cudaSuccess || units < 1)
      return tp_cuda(ctx, e ? e : cudaErrorInvalidConfiguration, "cov cluster occupancy");
  }
  if (ctx->max_ctas > 0 && units * CS > ctx->max_ctas) units = std::max(1, ctx->max_ctas / CS);
  if (units > njobs) units = njobs;
  // the grid is trimmed so that the region stores stay within 64 GB of HBM
  size_t slot = Slot<DIM, 1>::bytes(cap);
  const size_t budget = size_t(64) << 30;
  if ((size_t)units * slot > budget) units = std::max(1, (int)(budget / slot));
  int st = ctx->ensure_scratch((size_t)units * slot);
  if (st) return st;
  EngineCfg cfg{0.0, rel_tol, TP_NORM_L1, cap, 4000};
  e = cudaMemsetAsync(ctx->d_counter, 0, sizeof(int), ctx->stream);
  if (e == cudaSuccess) {
    lc.gridDim = dim3(units * CS);
    e = cudaLaunchKernelEx(&lc, kern, pol, njobs, ctx->d_counter, cfg, ctx->d_scratch, slot);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return tp_cuda(ctx, e, "cov launch");
}

// CTA slots of the device for policy P with one CTA per integral
template <int DIM, class P>
inline int engine_slots(tp_ctx* ctx) {
  constexpr int NT = 256;
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  size_t smem = engine_smem_bytes<DIM, 1, P>();
  cudaFuncSetAttribute(k_cov<DIM, P, NT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cov<DIM, P, NT, 1>, NT, smem) != cudaSuccess)
    per_sm = 1;
  cudaGetLastError();
  return sms * std::max(per_sm, 1);
}

// cluster: 1 = one CTA per integral, 8 = one 8-CTA cluster per integral,
// 0 = 8 when the batch has no more integrals than the device has CTA slots
// (a smaller batch would leave SMs idle, and its most expensive integral
// would set the time), else 1; 16 = one 16-CTA cluster per integral when
// the batch fills no more than the CTA slots that way (policies with
// P::CLUSTER16), else as 8. A policy whose clusters do not fit runs with the
// next smaller form.
//
// cap: regions per integral; 0 = the covariance default (6-D square-window
// T1, oscillating 2-D T2 and the halo-model terms refine to 10^5 regions and
// more): at least 2^19.
template <int DIM, class P>
inline int run_engine(tp_ctx* ctx, const P& pol, int njobs, double rel_tol, int cluster = 0, int cap = 0) {
  constexpr int NT = 256;
  if (njobs == 0) return TP_OK;
  if (cap <= 0) cap = std::max(ctx->region_cap, 1 << 19);
  if (cluster == 0) cluster = njobs <= engine_slots<DIM, P>(ctx) ? 8 : 1;
  if constexpr (P::CLUSTER16) {
    if (cluster == 16) {
      if ((long)njobs * 16 <= (long)engine_slots<DIM, P>(ctx)) {
        const int st = run_engine_cs<DIM, P, 16>(ctx, pol, njobs, rel_tol, cap);
        if (st != TP_ERR_CUDA || ctx->err.find("cluster") == std::string::npos) return st;
        cudaGetLastError();  // no 16-CTA cluster fits: 8-CTA clusters
      }
      cluster = 8;
    }
  }
  if (cluster == 8) {
    const int st = run_engine_cs<DIM, P, 8>(ctx, pol, njobs, rel_tol, cap);
    if (st != TP_ERR_CUDA || ctx->err.find("cluster occupancy") == std::string::npos) return st;
    cudaGetLastError();  // no 8-CTA cluster of this policy fits: one CTA per integral
  }
  return run_engine_cs<DIM, P, 1>(ctx, pol, njobs, rel_tol, cap);
}

// Integrates jobs[i] with policy pol (its jobs / out / status pointers are
// set here) into res[i]. Integrals that stop at the region cap are integrated
// again from the start with 16x the cap, up to ctx->escalate_cap regions (the
// reference's hcubature_v has no cap; the region sequence up to the old cap
// is the same, so an escalated value is the uncapped one); bad counts the
// integrals left at a cap or the sweep limit.
//
// first_cap: regions of the first pass (0 = the covariance default, at least
// 2^19). A small first cap sends the few expensive integrals of a batch to
// the later passes, which hold few integrals and so run on larger clusters.
template <int DIM, class P>
inline int run_jobs(tp_ctx* ctx, P pol, const std::vector<CovJob>& jobs, double rel_tol, int cluster,
                    std::vector<double>& res, int& bad, int first_cap = 0) {
  const size_t n = jobs.size();
  res.assign(n, 0.0);
  if (n == 0) return TP_OK;
  std::vector<CovJob> cur = jobs;
  std::vector<int> where(n);
  for (size_t i = 0; i < n; ++i) where[i] = (int)i;
  int cap = first_cap > 0 ? first_cap : std::max(ctx->region_cap, 1 << 19);
  for (;;) {
    const size_t m = cur.size();
    const size_t o_o = (sizeof(CovJob) * m + 255) & ~size_t(255);
    const size_t o_s = o_o + ((sizeof(double) * m + 255) & ~size_t(255));
    int st = ctx->ensure_io(o_s + sizeof(int) * m + 256);
    if (st) return st;
    char* b = ctx->d_io;
    cudaError_t e = cudaMemcpyAsync(b, cur.data(), sizeof(CovJob) * m, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return tp_cuda(ctx, e, "cov upload");
    pol.jobs = (const CovJob*)b;
    pol.out = (double*)(b + o_o);
    pol.status = (int*)(b + o_s);
    st = run_engine<DIM>(ctx, pol, (int)m, rel_tol, cluster, cap);
    if (st) return st;
    std::vector<double> v(m);
    std::vector<int> hs(m);
    e = cudaMemcpy(v.data(), b + o_o, sizeof(double) * m, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(hs.data(), b + o_s, sizeof(int) * m, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return tp_cuda(ctx, e, "cov download");
    const int next_cap = (int)std::min<long long>(16LL * cap, ctx->escalate_cap);
    std::vector<CovJob> again;
    std::vector<int> again_at;
    for (size_t i = 0; i < m; ++i) {
      res[where[i]] = v[i];
      if ((hs[i] & 1) && next_cap > cap) {
        again.push_back(cur[i]);
        again_at.push_back(where[i]);
      } else if (hs[i]) {
        ++bad;
      }
    }
    if (again.empty()) return TP_OK;
    cur.swap(again);
    where.swap(again_at);
    cap = next_cap;
  }
}

}  // namespace tp
