// Gaussian likelihood of <Map^3> model vectors, the consumer of the module's
// output (cosmosis/threepoint_likelihood.py:8-58 of the reference):
// chi2 = (m - d)^T C^-1 (m - d), log L = -chi2 / 2 (the reference sets its
// log-determinant term to 0).
//
// Set-up factors the covariance once on the GPU (FP64 Cholesky C = L L^T,
// then L^-1 and C^-1 = L^-T L^-1); every evaluation is chi2 = |L^-1 (m - d)|^2,
// one CTA per model vector, so a whole batch of cosmologies is one launch.
// The reference inverts C with numpy (LU); for a covariance (symmetric
// positive definite) both give the same chi2 to rounding, and a matrix that is
// not positive definite is rejected here.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "threepoint_gb300.h"

namespace {

constexpr int LNT = 1024;  // threads of the factorisation CTA
constexpr int CNT = 256;   // threads per chi2 CTA

// In-place lower Cholesky of a (n x n, row-major; the lower triangle is read),
// then X = L^-1 (lower) and inv = X^T X. One CTA; *status = 1 + column of the
// first non-positive pivot, or 0.
__global__ void __launch_bounds__(LNT) k_chol_inverse(double* a, double* x, double* inv, int n, int* status) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    // a[j][j] has received every update from columns < j
    const double d = a[(size_t)j * n + j];
    if (!(d > 0.0)) {
      if (threadIdx.x == 0) bad = j + 1;
      break;
    }
    const double ld = sqrt(d);
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) a[(size_t)i * n + j] /= ld;
    if (threadIdx.x == 0) a[(size_t)j * n + j] = ld;
    __syncthreads();
    // trailing update of the lower triangle: a[i][k] -= l[i][j] l[k][j], j < k <= i
    const long m = n - j - 1;
    const long cnt = m * (m + 1) / 2;
    for (long t = threadIdx.x; t < cnt; t += blockDim.x) {
      // t -> (r, c) with 0 <= c <= r < m, row-major over the lower triangle
      long r = (long)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
      while (r * (r + 1) / 2 > t) --r;
      while ((r + 1) * (r + 2) / 2 <= t) ++r;
      const long c = t - r * (r + 1) / 2;
      const int i = j + 1 + (int)r, k = j + 1 + (int)c;
      a[(size_t)i * n + k] -= a[(size_t)i * n + j] * a[(size_t)k * n + j];
    }
    __syncthreads();
  }
  __syncthreads();
  if (bad) {
    if (threadIdx.x == 0) *status = bad;
    return;
  }
  // X = L^-1 by forward substitution, one column of X per thread
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    for (int i = 0; i < n; ++i) {
      double s = (i == c) ? 1.0 : 0.0;
      for (int k = c; k < i; ++k) s -= a[(size_t)i * n + k] * x[(size_t)k * n + c];
      x[(size_t)i * n + c] = (i < c) ? 0.0 : s / a[(size_t)i * n + i];
    }
  }
  __syncthreads();
  // inv = X^T X
  for (long t = threadIdx.x; t < (long)n * n; t += blockDim.x) {
    const int r = (int)(t / n), c = (int)(t % n);
    const int k0 = r > c ? r : c;
    double s = 0.0;
    for (int k = k0; k < n; ++k) s += x[(size_t)k * n + r] * x[(size_t)k * n + c];
    inv[t] = s;
  }
  if (threadIdx.x == 0) *status = 0;
}

// chi2 of model vector b (row b of models, leading dimension ld):
// z = X (m - d), chi2 = sum z_i^2, summed in a fixed order.
__global__ void __launch_bounds__(CNT) k_chi2(const double* x, const double* data, const double* models, long ld,
                                              int n, double* chi2) {
  extern __shared__ double sm[];
  double* r = sm;          // [n]
  double* part = sm + n;   // [CNT]
  const double* m = models + (size_t)blockIdx.x * ld;
  for (int i = threadIdx.x; i < n; i += blockDim.x) r[i] = m[i] - data[i];
  __syncthreads();
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double z = 0.0;
    const double* xi = x + (size_t)i * n;
    for (int k = 0; k <= i; ++k) z += xi[k] * r[k];
    acc += z * z;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int o = CNT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) chi2[blockIdx.x] = part[0];
}

}  // namespace

struct tp_likelihood {
  int device = 0;
  int n = 0;
  cudaStream_t stream = nullptr;
  double* d_x = nullptr;     // L^-1
  double* d_inv = nullptr;   // C^-1
  double* d_data = nullptr;  // measured vector
  double* d_io = nullptr;    // host-API staging
  size_t io_bytes = 0;
  std::string err;
};

static int lk_cuda(tp_likelihood* lk, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return TP_OK;
  if (lk) lk->err = std::string(where) + ": " + cudaGetErrorString(e);
  return TP_ERR_CUDA;
}

extern "C" const char* tp_likelihood_last_error(const tp_likelihood* lk) { return lk ? lk->err.c_str() : "null"; }

extern "C" void tp_likelihood_destroy(tp_likelihood* lk) {
  if (!lk) return;
  cudaSetDevice(lk->device);
  cudaFree(lk->d_x);
  cudaFree(lk->d_inv);
  cudaFree(lk->d_data);
  cudaFree(lk->d_io);
  if (lk->stream) cudaStreamDestroy(lk->stream);
  delete lk;
}

extern "C" int tp_likelihood_create(int device, const double* data, const double* cov, int n, tp_likelihood** out) {
  if (!out || !data || !cov || n < 1 || n > 8192) return TP_ERR_ARG;
  *out = nullptr;
  for (long i = 0; i < (long)n * n; ++i)
    if (!std::isfinite(cov[i])) return TP_ERR_ARG;
  tp_likelihood* lk = new tp_likelihood();
  lk->device = device;
  lk->n = n;
  cudaError_t e = cudaSetDevice(device);
  const size_t nn = (size_t)n * n * sizeof(double);
  double* d_a = nullptr;
  int* d_st = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&lk->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&lk->d_x, nn);
  if (e == cudaSuccess) e = cudaMalloc(&lk->d_inv, nn);
  if (e == cudaSuccess) e = cudaMalloc(&lk->d_data, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d_a, nn);
  if (e == cudaSuccess) e = cudaMalloc(&d_st, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_a, cov, nn, cudaMemcpyHostToDevice, lk->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lk->d_data, data, sizeof(double) * n, cudaMemcpyHostToDevice, lk->stream);
  if (e == cudaSuccess) {
    k_chol_inverse<<<1, LNT, 0, lk->stream>>>(d_a, lk->d_x, lk->d_inv, n, d_st);
    e = cudaGetLastError();
  }
  int st = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, d_st, sizeof(int), cudaMemcpyDeviceToHost, lk->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(lk->stream);
  cudaFree(d_a);
  cudaFree(d_st);
  if (e != cudaSuccess) {
    tp_likelihood_destroy(lk);
    return TP_ERR_CUDA;
  }
  if (st != 0) {  // not positive definite
    tp_likelihood_destroy(lk);
    return TP_ERR_ARG;
  }
  *out = lk;
  return TP_OK;
}

extern "C" int tp_likelihood_cov_inv(tp_likelihood* lk, double* out) {
  if (!lk || !out) return TP_ERR_ARG;
  cudaSetDevice(lk->device);
  cudaError_t e = cudaMemcpyAsync(out, lk->d_inv, sizeof(double) * lk->n * lk->n, cudaMemcpyDeviceToHost, lk->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(lk->stream);
  return lk_cuda(lk, e, "cov_inv");
}

extern "C" int tp_likelihood_chi2_device(tp_likelihood* lk, const double* models_device, int n_models, long ld,
                                         double* chi2_device, void* stream) {
  if (!lk || !models_device || !chi2_device || n_models < 0 || ld < lk->n) return TP_ERR_ARG;
  if (n_models == 0) return TP_OK;
  cudaSetDevice(lk->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : lk->stream;
  const size_t smem = sizeof(double) * (lk->n + CNT);
  if (smem > 200 * 1024) return TP_ERR_ARG;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_chi2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return lk_cuda(lk, e, "chi2 attribute");
  }
  k_chi2<<<n_models, CNT, smem, s>>>(lk->d_x, lk->d_data, models_device, ld, lk->n, chi2_device);
  return lk_cuda(lk, cudaGetLastError(), "chi2 launch");
}

extern "C" int tp_likelihood_chi2(tp_likelihood* lk, const double* models, int n_models, double* chi2_out) {
  if (!lk || !models || !chi2_out || n_models < 0) return TP_ERR_ARG;
  if (n_models == 0) return TP_OK;
  cudaSetDevice(lk->device);
  const size_t in = sizeof(double) * (size_t)n_models * lk->n, outb = sizeof(double) * (size_t)n_models;
  const size_t need = ((in + 255) & ~size_t(255)) + outb;
  cudaError_t e = cudaSuccess;
  if (need > lk->io_bytes) {
    cudaFree(lk->d_io);
    lk->d_io = nullptr;
    lk->io_bytes = 0;
    e = cudaMalloc(&lk->d_io, need);
    if (e != cudaSuccess) return lk_cuda(lk, e, "chi2 staging");
    lk->io_bytes = need;
  }
  double* d_m = lk->d_io;
  double* d_c = (double*)((char*)lk->d_io + ((in + 255) & ~size_t(255)));
  e = cudaMemcpyAsync(d_m, models, in, cudaMemcpyHostToDevice, lk->stream);
  if (e != cudaSuccess) return lk_cuda(lk, e, "chi2 upload");
  int st = tp_likelihood_chi2_device(lk, d_m, n_models, lk->n, d_c, nullptr);
  if (st) return st;
  e = cudaMemcpyAsync(chi2_out, d_c, outb, cudaMemcpyDeviceToHost, lk->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(lk->stream);
  return lk_cuda(lk, e, "chi2");
}
