// Launch descriptors and device utilities shared between the kernel
// translation units and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tp_internal.cuh"

namespace tp {

// ---- bulk async copy global -> shared with an mbarrier (bounded wait) -----
struct BulkBar {
  unsigned long long bar;
  unsigned phase;
  unsigned timeouts;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// thread 0 only, once per CTA before the first copy
__device__ __forceinline__ void bulkbar_init(BulkBar* b) {
  uint32_t a = smem_u32(&b->bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  b->phase = 0;
  b->timeouts = 0;
}

// thread 0 only: copies bytes (multiple of 16, both addresses 16-byte aligned)
// with cp.async.bulk and waits for completion with an iteration cap. Returns
// false (and counts a timeout) if the cap was reached.
__device__ __forceinline__ bool bulk_copy_g2s(BulkBar* b, void* dst, const void* src, unsigned bytes) {
  uint32_t a = smem_u32(&b->bar), d = smem_u32(dst);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
               "l"(src), "r"(bytes), "r"(a)
               : "memory");
  const uint32_t ph = b->phase;
  uint32_t ok = 0;
  for (int it = 0; it < (1 << 22) && !ok; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(ph)
        : "memory");
  }
  b->phase = ph ^ 1u;
  if (!ok) b->timeouts++;
  return ok != 0;
}

// ---- Map3 launch ------------------------------------------------------------
struct Map3Launch {
  int precision;
  int njobs;
  const int* job_cosmo;     // device [njobs]
  const double* job_theta;  // device [njobs][3]
  const double* ncoef64;    // device node coefficients (FP64, weight column normalised)
  const float* ncoef32;
  const float* fcoef32;  // NF_* rows, read by the FP32 kernel
  const double* wscale64;   // device [n_cosmo] weight scales
  const double* wscale32;
  const void* ck64;         // device CosmoK<double>[n_cosmo]
  const void* ck32;         // device CosmoK<float>[n_cosmo]
  double lmin, lmax, phimin, phimax, rel_tol;
  int cap, max_sweeps;
  double* out;
  double* err;
  int64_t* neval;
  int64_t* nlive;
  int* status;
  const int* job_order;  // optional device permutation of the job indices
  int* job_counter;  // device int
  unsigned* diag;    // device counter of bulk-copy timeouts (may be null)
  int cluster = 1;   // CTAs per integral (1, or 8 from plan_map3)
};

// shared memory that the resident CTAs of k_map3<float> hold on one SM
// (dynamic + per-block reserved)
cudaError_t map3_f32_resident_smem(size_t* bytes);

// grid size, dynamic shared memory and scratch bytes of a Map3 launch
// Launch plan of k_map3: grid, CTAs per integral (1, or 8 when allow_cluster
// and the batch has no more integrals than CTA slots), dynamic shared memory
// per CTA and the scratch bytes of the region stores.
cudaError_t plan_map3(int precision, int njobs, int cap, int max_ctas, int allow_cluster, int* grid, int* cluster,
                      size_t* smem, size_t* scratch);
cudaError_t launch_map3(const Map3Launch& L, int grid, size_t smem, char* scratch, cudaStream_t st);

cudaError_t launch_bkappa_points(int precision, const int* cosmo_idx, const double* ell, long n, const void* ncoef,
                                 const double* wscale, const void* ck, double* out, cudaStream_t st);
cudaError_t launch_bkappa_nodes(int precision, int cosmo, const double* ell, long n, const void* ncoef,
                                const double* wscale, const void* ck, double* term, double* bis, cudaStream_t st);

}  // namespace tp
