// Context object behind the opaque tp_ctx handle (host side).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>
#include <unordered_map>
#include <vector>

#include "tp_internal.cuh"

// NVTX range over one entry-point call (host time: the table build, the
// integral launches and their synchronisation), visible in Nsight tools;
// NVTX is header-only and costs nothing without a profiler attached.
struct TpRange {
  explicit TpRange(const char* name) { nvtxRangePushA(name); }
  ~TpRange() { nvtxRangePop(); }
  TpRange(const TpRange&) = delete;
  TpRange& operator=(const TpRange&) = delete;
};

struct tp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int max_ctas = 0;        // 0 = all resident CTAs
  int region_cap = 32768;  // regions per adaptive integral
  // integrals of the host-API calls that reach region_cap are integrated
  // again with 16x the cap, up to this many regions (the reference's
  // hcubature_v has no cap); <= region_cap turns this off
  int escalate_cap = 1 << 24;

  // cosmologies and their device tables
  int n_cosmo = 0;
  int cosmo_cap = 0;
  size_t nz_cap = 0;
  std::vector<tp::CosmoDev> h_cos;
  tp::CosmoDev* d_cos = nullptr;
  tp::EHConst* d_eh = nullptr;
  tp::TablesDev* d_tab = nullptr;
  double* d_nz = nullptr;
  double* d_ncoef64 = nullptr;
  float* d_ncoef32 = nullptr;
  float* d_fcoef32 = nullptr;  // NF_* rows of the FP32 point path
  double* d_hcoef = nullptr;
  float* d_hcoef32 = nullptr;
  double* d_wscale64 = nullptr;
  double* d_wscale32 = nullptr;
  void* d_ck64 = nullptr;
  void* d_ck32 = nullptr;
  float4* d_plt = nullptr;  // [n_cosmo][PLT_N] log2 P_lin cubic segments
  double* d_ehg = nullptr;  // [n_cosmo][EHG_N] 2 ln T(k) of the sigma(R) integrand
  // halo-model tables (covariance terms T5-T7), built per cosmology on first use
  tp::HaloTab* d_halo = nullptr;
  std::vector<char> halo_ready;
  // CTAs that share one T5-T7 integral (a thread-block cluster): 16 (16 when
  // the batch leaves room for that many per integral, else 8), 8 or 1
  int halo_cluster = 16;
  // <Map^3> host calls with no more integrals than CTA slots run one 8-CTA
  // cluster per integral (0: always one CTA per integral)
  int map3_cluster = 1;
  // relative tolerance of the T5, T6, T7 integrals (index 5..7); 0 = the reference's
  double cov_rel_tol[8] = {0, 0, 0, 0, 0, 0, 0, 0};

  // shape noise of P(ell)
  double sigma_eps = 0.0, ngal = 1.0;
  int constant_ps = 0;
  // second side of a rectangular survey [rad]; 0 = not set
  double theta_max_smaller = 0.0;

  // scratch: per-CTA region stores; io: staging of host-API inputs/outputs
  char* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  char* d_io = nullptr;
  size_t io_bytes = 0;
  // expected cost (cubature points) of each <Map^3> integral seen so far,
  // keyed by triplet and settings; orders later launches longest-first
  std::unordered_map<std::string, double> map3_cost;
  int* d_counter = nullptr;
  unsigned* d_diag = nullptr;

  void free_cosmo();
  int ensure_scratch(size_t bytes);
  int ensure_io(size_t bytes);
};

int tp_fail(tp_ctx* ctx, int st, const std::string& msg);
int tp_cuda(tp_ctx* ctx, cudaError_t e, const char* where);
