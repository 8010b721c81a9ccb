// Allocation-free variant of the batched <Map^3> launch.
//
// Some callers cannot allocate device memory at the time they integrate: code
// running while a CUDA stream is being captured into a graph (cudaMalloc is
// not a capturable operation), callers that run under a memory pool or a
// framework allocator that owns every device allocation, and real-time
// pipelines that forbid allocation after start-up. tp_map3_jobs_noalloc
// serves them: it allocates nothing and keeps the per-CTA region stores in
// the fixed-size device array below instead of context scratch.
//
// The array is a file-scope __device__ object of TP_NOALLOC_SCRATCH_BYTES: it
// exists on every GPU that loads this library until the process exits. Every
// call shares it (and the job counter next to it), so calls that overlap on
// the GPU (two streams, two host threads) race and corrupt each other's
// results; serialise them. The array keeps the last call's contents; the only
// state that must start at zero, the job counter, is cleared by each call.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "tp_capi_internal.h"
#include "tp_cubature.cuh"
#include "tp_kernels.cuh"

// 128 MiB: 192 CTAs of 8192-region stores (696,576 bytes each) for the 3-D
// <Map^3> integrals
#define TP_NOALLOC_SCRATCH_BYTES (128u << 20)
#define TP_NOALLOC_REGION_CAP 8192
#define TP_NOALLOC_MAX_DEVICES 64
static_assert(TP_NOALLOC_SCRATCH_BYTES / tp::Slot<3, 1>::bytes(TP_NOALLOC_REGION_CAP) == 192,
              "the array holds 192 region stores of the cap");

static __device__ __align__(256) char g_noalloc_scratch[TP_NOALLOC_SCRATCH_BYTES];
static __device__ __align__(256) int g_noalloc_counter[64];

namespace {
struct NoallocDevice {
  bool ready = false;
  char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int* counter = nullptr;   // device address of g_noalloc_counter on this device
};
NoallocDevice g_dev[TP_NOALLOC_MAX_DEVICES];

std::mutex g_setup_mutex;

// Once per device, with that device current: the host-side names of the
// __device__ arrays are only stand-ins, so their device addresses are looked
// up here and passed to the kernel. First calls from two host threads are
// serialised by the mutex.
int noalloc_setup(tp_ctx* ctx) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  NoallocDevice& d = g_dev[ctx->device];
  if (d.ready) return TP_OK;
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "no-alloc scratch address");
  d.scratch = (char*)p;
  e = cudaGetSymbolAddress(&p, g_noalloc_counter);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "no-alloc counter address");
  d.counter = (int*)p;
  d.ready = true;
  return TP_OK;
}
}  // namespace

using namespace tp;

extern "C" int tp_map3_jobs_noalloc(tp_ctx* ctx, const int* job_cosmo_device, const double* job_theta_device,
                                    int n_jobs, double phi_min, double phi_max, double l_min, double l_max,
                                    double rel_tol, int precision, double* out_device, double* err_device,
                                    int* status_device) {
  if (!ctx || !job_cosmo_device || !job_theta_device || !out_device || n_jobs < 0) return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  if (!(rel_tol > 0) || !(phi_max > phi_min) || !(l_min >= 0)) return TP_ERR_ARG;
  if (ctx->n_cosmo == 0) return tp_fail(ctx, TP_ERR_STATE, "no cosmology set");
  if (ctx->device < 0 || ctx->device >= TP_NOALLOC_MAX_DEVICES) return tp_fail(ctx, TP_ERR_ARG, "device index");
  if (n_jobs == 0) return TP_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "set device");
  int st = noalloc_setup(ctx);
  if (st) return st;
  int grid = 0, cluster = 1;
  size_t smem = 0, need = 0;
  e = plan_map3(precision, n_jobs, TP_NOALLOC_REGION_CAP, ctx->max_ctas, 0, &grid, &cluster, &smem, &need);
  if (e != cudaSuccess) return tp_cuda(ctx, e, "no-alloc plan");
  // the persistent grid is trimmed to the CTAs whose region stores fit the array
  const size_t slot = need / (size_t)grid;
  const int fit = (int)(TP_NOALLOC_SCRATCH_BYTES / slot);
  if (fit < 1) return tp_fail(ctx, TP_ERR_CAPACITY, "no-alloc scratch smaller than one region store");
  if (grid > fit) grid = fit;
  if ((size_t)grid * slot > TP_NOALLOC_SCRATCH_BYTES)
    return tp_fail(ctx, TP_ERR_CAPACITY, "no-alloc launch exceeds the " + std::to_string(TP_NOALLOC_SCRATCH_BYTES) +
                                             "-byte scratch array");
  const NoallocDevice& d = g_dev[ctx->device];
  Map3Launch L;
  L.precision = precision;
  L.njobs = n_jobs;
  L.job_cosmo = job_cosmo_device;
  L.job_theta = job_theta_device;
  L.ncoef64 = ctx->d_ncoef64;
  L.ncoef32 = ctx->d_ncoef32;
  L.fcoef32 = ctx->d_fcoef32;
  L.wscale64 = ctx->d_wscale64;
  L.wscale32 = ctx->d_wscale32;
  L.ck64 = ctx->d_ck64;
  L.ck32 = ctx->d_ck32;
  L.lmin = l_min;
  L.lmax = l_max;
  L.phimin = phi_min;
  L.phimax = phi_max;
  L.rel_tol = rel_tol;
  L.cap = TP_NOALLOC_REGION_CAP;
  L.max_sweeps = 2000;
  L.out = out_device;
  L.err = err_device;
  L.neval = nullptr;
  L.nlive = nullptr;
  L.status = status_device;
  L.job_counter = d.counter;  // cleared by launch_map3 (cudaMemsetAsync) before the kernel
  L.diag = ctx->d_diag;  // allocated with the context: bulk-copy timeouts are counted as in tp_map3_jobs_device
  L.job_order = nullptr;
  e = launch_map3(L, grid, smem, d.scratch, ctx->stream);
  return tp_cuda(ctx, e, "no-alloc map3 launch");
}
