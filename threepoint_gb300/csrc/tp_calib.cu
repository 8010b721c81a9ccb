// Micro-benchmarks of the pipes that bound the integrand kernels: the SFU
// (MUFU ex2.approx.f32) and the FP32/FP64 FMA pipes. Used to report the
// roofline denominators of the compute-bound kernels, whose algorithmic work
// is counted in SFU operations and FMAs rather than bytes.
#include <cuda_runtime.h>

#include "tp_capi_internal.h"

namespace {

__global__ void k_sfu(float* out, int iters) {
  float a0 = threadIdx.x * 1e-3f, a1 = a0 + 0.1f, a2 = a0 + 0.2f, a3 = a0 + 0.3f;
  float a4 = a0 + 0.4f, a5 = a0 + 0.5f, a6 = a0 + 0.6f, a7 = a0 + 0.7f;
  for (int i = 0; i < iters; ++i) {
#define EX2(x) asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x))
    EX2(a0); EX2(a1); EX2(a2); EX2(a3); EX2(a4); EX2(a5); EX2(a6); EX2(a7);
#undef EX2
  }
  if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == 12345.f) out[0] = a0;
}

template <typename T>
__global__ void k_fma(T* out, int iters) {
  T a0 = threadIdx.x * (T)1e-3, a1 = a0 + (T)0.1, a2 = a0 + (T)0.2, a3 = a0 + (T)0.3;
  T a4 = a0 + (T)0.4, a5 = a0 + (T)0.5, a6 = a0 + (T)0.6, a7 = a0 + (T)0.7;
  const T m = (T)0.9999, c = (T)1e-4;
  for (int i = 0; i < iters; ++i) {
    a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
    a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
  }
  if (a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7 == (T)12345) out[0] = a0;
}

template <typename K>
double time_kernel(K kern, int blocks, int threads, double ops) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kern(blocks, threads);  // warm-up
  cudaEventRecord(e0);
  kern(blocks, threads);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ops / (ms * 1e-3);
}

}  // namespace

// out[0] = ex2.approx.f32 per second, out[1] = FP32 FMA per second,
// out[2] = FP64 FMA per second (whole device, measured now).
extern "C" int tp_pipe_peaks(int device, double* out) {
  if (!out) return TP_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return TP_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  float* buf = nullptr;
  if (cudaMalloc((void**)&buf, 64) != cudaSuccess) return TP_ERR_CUDA;
  const int threads = 256, blocks = sms * 8;
  const int it_sfu = 4096, it_fma = 8192, it_d = 1024;
  out[0] = time_kernel([&](int b, int t) { k_sfu<<<b, t>>>(buf, it_sfu); }, blocks, threads,
                       8.0 * it_sfu * (double)blocks * threads);
  out[1] = time_kernel([&](int b, int t) { k_fma<float><<<b, t>>>(buf, it_fma); }, blocks, threads,
                       8.0 * it_fma * (double)blocks * threads);
  out[2] = time_kernel([&](int b, int t) { k_fma<double><<<b, t>>>((double*)buf, it_d); }, blocks, threads,
                       8.0 * it_d * (double)blocks * threads);
  cudaError_t e = cudaDeviceSynchronize();
  cudaFree(buf);
  return e == cudaSuccess ? TP_OK : TP_ERR_CUDA;
}

extern "C" void* tp_ctx_stream(tp_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
