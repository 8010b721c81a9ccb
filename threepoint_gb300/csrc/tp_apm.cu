// FFT aperture-mass measurement on the GPU: shear catalogue -> cloud-in-cell
// grids -> aperture-mass maps M_ap(theta) by zero-padded FFT convolution with
// the Q filter -> <Map^3> of every theta triplet over the map interiors.
//
// Reference: python_scripts/aperture_mass_computer.py: the class
// aperture_mass_computer (Qfunc/Qfunc_array :82-106, Map_fft with a weight
// grid and normalize_weighted :199-286, norm_fft :283-286, normalize_shear
// with CIC :288-372) and extract_Map3 / extract_Map3_of_field (:375-531).
//
// Design: one tp_apm object per (grid size, field size, apertures, filter)
// keeps on the device the FFTs of the three filter grids of every aperture
// (Re Q, Im Q and |Q| zero-padded to F x F, F >= 2 npix - 1), computed once,
// so a field costs three forward transforms (the shear grid's real and
// imaginary parts and the weight grid) and two inverse ones per aperture
// (numerator Im(g) * Im(Q) - Re(g) * Re(Q) and denominator w * |Q| multiplied
// in Fourier space by one fused kernel). The 2-D FFTs are cuFFT's (loaded at
// run time with dlopen so that the rest of the library does not depend on
// it), in FP64 (TP_FP64, the reference's numpy precision) or FP32 (TP_FP32:
// transforms, filter spectra and Fourier products in FP32; gridding, maps and
// the triplet sums stay FP64); gridding, filters, spectral products, the
// crop/divide and the triplet reduction are this file's kernels. The triplet
// reduction reads each pixel's n_theta map values once and accumulates all
// triplets.
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "tp_capi_internal.h"

namespace {

// ---- cuFFT through dlopen --------------------------------------------------
struct CufftApi {
  bool ok = false;
  std::string why;
  cufftResult (*plan2d)(cufftHandle*, int, int, cufftType) = nullptr;
  cufftResult (*exec_d2z)(cufftHandle, cufftDoubleReal*, cufftDoubleComplex*) = nullptr;
  cufftResult (*exec_z2d)(cufftHandle, cufftDoubleComplex*, cufftDoubleReal*) = nullptr;
  cufftResult (*exec_r2c)(cufftHandle, cufftReal*, cufftComplex*) = nullptr;
  cufftResult (*exec_c2r)(cufftHandle, cufftComplex*, cufftReal*) = nullptr;
  cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
  cufftResult (*destroy)(cufftHandle) = nullptr;
};

const CufftApi& cufft() {
  static CufftApi api;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libcufft.so.12", "libcufft.so.11", "libcufft.so"};
    void* h = nullptr;
    for (const char* n : names)
      if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
      api.why = "libcufft not found (dlopen)";
      return;
    }
    api.plan2d = (decltype(api.plan2d))dlsym(h, "cufftPlan2d");
    api.exec_d2z = (decltype(api.exec_d2z))dlsym(h, "cufftExecD2Z");
    api.exec_z2d = (decltype(api.exec_z2d))dlsym(h, "cufftExecZ2D");
    api.exec_r2c = (decltype(api.exec_r2c))dlsym(h, "cufftExecR2C");
    api.exec_c2r = (decltype(api.exec_c2r))dlsym(h, "cufftExecC2R");
    api.set_stream = (decltype(api.set_stream))dlsym(h, "cufftSetStream");
    api.destroy = (decltype(api.destroy))dlsym(h, "cufftDestroy");
    api.ok = api.plan2d && api.exec_d2z && api.exec_z2d && api.exec_r2c && api.exec_c2r && api.set_stream &&
             api.destroy;
    if (!api.ok) api.why = "libcufft lacks a needed symbol";
  });
  return api;
}

// smallest size >= n whose prime factors are 2, 3, 5 and 7
int fft_size(int n) {
  for (int m = n;; ++m) {
    int r = m;
    for (int p : {2, 3, 5, 7})
      while (r % p == 0) r /= p;
    if (r == 1) return m;
  }
}

constexpr double PI = 3.14159265358979323846;

// ---- kernels ----------------------------------------------------------------

// Cloud-in-cell gridding (normalize_shear, CIC, aperture_mass_computer.py:
// 318-367): every galaxy adds its shear and weight, times the bilinear
// weights of its cell position x / (fieldsize / (npix - 1)), to the four bins
// that numpy.histogram2d assigns to (x, y), (x + cell, y), (x, y + cell) and
// (x + cell, y + cell) over the bin edges e_i = i / (npix - 1) * fieldsize,
// i = 0..npix (a value equal to the last edge falls into the last bin; values
// outside [e_0, e_npix] are dropped). Grids are row-major [x bin][y bin].
__device__ __forceinline__ int hist_bin(double v, const double* __restrict__ edges, int npix, double cell) {
  if (!(v >= edges[0] && v <= edges[npix])) return -1;
  if (v == edges[npix]) return npix - 1;
  int k = (int)floor(v / cell);
  k = k < 0 ? 0 : (k > npix - 1 ? npix - 1 : k);
  for (int it = 0; it < 3 && k > 0 && edges[k] > v; ++it) --k;
  for (int it = 0; it < 3 && k < npix - 1 && edges[k + 1] <= v; ++it) ++k;
  return k;
}

__global__ void k_apm_cic(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ g1,
                          const double* __restrict__ g2, long n, const double* __restrict__ edges, int npix,
                          double cell, double* sre, double* sim, double* nrm) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xv = x[i], yv = y[i], a = g1[i], b = g2[i];
  const double fx = xv / cell, fy = yv / cell;
  const double dx = fx - floor(fx), dy = fy - floor(fy);
  const double wx[2] = {1 - dx, dx}, wy[2] = {1 - dy, dy};
  const double ox[2] = {xv, xv + cell}, oy[2] = {yv, yv + cell};
#pragma unroll
  for (int cx = 0; cx < 2; ++cx) {
    const int bx = hist_bin(ox[cx], edges, npix, cell);
    if (bx < 0) continue;
#pragma unroll
    for (int cy = 0; cy < 2; ++cy) {
      const int by = hist_bin(oy[cy], edges, npix, cell);
      if (by < 0) continue;
      const double w = wx[cx] * wy[cy];
      const size_t o = (size_t)bx * npix + by;
      atomicAdd(&sre[o], a * w);
      atomicAdd(&sim[o], b * w);
      atomicAdd(&nrm[o], w);
    }
  }
}

// Q filter grid of one aperture (Qfunc_array, :82-106): at pixel (i, j),
// z = (i - npix/2) + I (j - npix/2), r = |z| fieldsize / npix,
// q = Q(r) conj(z)^2 / |z|^2 (0 at z = 0) with Q the exponential filter
// (r/t)^2 / (4 pi t^2) exp(-(r/t)^2 / 2) or the polynomial one
// 6 / pi (r/t)^4 (1 - (r/t)^4) / t^2 inside r <= t. Writes Re q, Im q and |q|
// into the top-left npix x npix corner of three zero-padded F x F grids
// (computed in FP64, stored in T).
template <typename T>
__global__ void k_apm_filter(int npix, int F, double fieldsize, double theta, int polynomial, T* qr, T* qi, T* qa) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)npix * npix) return;
  const int i = (int)(t / npix), j = (int)(t % npix);
  const double zr = i - npix / 2.0, zi = j - npix / 2.0;
  const double z2 = zr * zr + zi * zi;
  const double r = sqrt(z2) * fieldsize / npix;
  double re = 0, im = 0, ab = 0;
  if (r != 0) {
    const double th2 = (r / theta) * (r / theta);
    double Q;
    if (polynomial)
      Q = th2 > 1 ? 0.0 : 6 / PI * th2 * th2 * (1. - th2 * th2) / (theta * theta);
    else
      Q = th2 / (4 * PI * theta * theta) * exp(-th2 / 2);
    // conj(z)^2 / |z|^2 = (zr^2 - zi^2 - 2 I zr zi) / |z|^2
    re = Q * (zr * zr - zi * zi) / z2;
    im = Q * (-2 * zr * zi) / z2;
    ab = sqrt(re * re + im * im);
  }
  const size_t o = (size_t)i * F + j;
  qr[o] = (T)re;
  qi[o] = (T)im;
  qa[o] = (T)ab;
}

// U filter grid of one aperture (Ufunc/Ufunc_array, :72-114), exponential
// filter: U(r) = exp(-x) (1 - x) / (2 pi theta^2), x = (r/theta)^2 / 2
template <typename T>
__global__ void k_apm_ufilter(int npix, int F, double fieldsize, double theta, T* u) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)npix * npix) return;
  const int i = (int)(t / npix), j = (int)(t % npix);
  const double zr = i - npix / 2.0, zi = j - npix / 2.0;
  const double r = sqrt(zr * zr + zi * zi) * fieldsize / npix;
  const double xh = (r / theta) * (r / theta) / 2;
  u[(size_t)i * F + j] = (T)(exp(-xh) * (1. - xh) / (2 * PI) / (theta * theta));
}

// spectrum product a * b (complex, C = double2 or float2), n entries
template <typename C>
__global__ void k_apm_mul(const C* __restrict__ a, const C* __restrict__ b, long n, C* c) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const C x = a[t], y = b[t];
  C r;
  r.x = x.x * y.x - x.y * y.y;
  r.y = x.x * y.y + x.y * y.x;
  c[t] = r;
}

// 'same'-mode window of an unnormalised inverse transform times scale
template <typename T>
__global__ void k_apm_crop_scaled(const T* __restrict__ v, int npix, int F, double scale, double* map) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)npix * npix) return;
  const int off = (npix - 1) / 2;
  const int i = (int)(t / npix), j = (int)(t % npix);
  map[t] = (double)v[(size_t)(i + off) * F + (j + off)] * scale;
}

// copies an npix x npix grid into the top-left corner of a zeroed F x F grid
template <typename T>
__global__ void k_apm_pad(const double* __restrict__ src, int npix, int F, T* dst) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)npix * npix) return;
  const int i = (int)(t / npix), j = (int)(t % npix);
  dst[(size_t)i * F + j] = (T)src[t];
}

// Fourier-space products of one aperture: num = Im(g) Im(Q) - Re(g) Re(Q),
// den = w |Q| (Map_fft :211-236 with norm_fft :283-286), cross (optional) =
// -(Re(g) Im(Q) + Im(g) Re(Q)) (return_mcross :246-255)
template <typename C>
__global__ void k_apm_spectra(const C* __restrict__ Yr, const C* __restrict__ Yi, const C* __restrict__ W,
                              const C* __restrict__ Qr, const C* __restrict__ Qi, const C* __restrict__ Qa, long n,
                              C* num, C* den, C* cross) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const C yr = Yr[t], yi = Yi[t], w = W[t], qr = Qr[t], qi = Qi[t], qa = Qa[t];
  C a, b;
  a.x = yi.x * qi.x - yi.y * qi.y - (yr.x * qr.x - yr.y * qr.y);
  a.y = yi.x * qi.y + yi.y * qi.x - (yr.x * qr.y + yr.y * qr.x);
  b.x = w.x * qa.x - w.y * qa.y;
  b.y = w.x * qa.y + w.y * qa.x;
  num[t] = a;
  den[t] = b;
  if (cross) {
    C c;
    c.x = -(yr.x * qi.x - yr.y * qi.y + yi.x * qr.x - yi.y * qr.y);
    c.y = -(yr.x * qi.y + yr.y * qi.x + yi.x * qr.y + yi.y * qr.x);
    cross[t] = c;
  }
}

// the 'same'-mode window of the linear convolution (rows and columns
// off .. off + npix - 1, off = (npix - 1) / 2): map = num / den (the inverse
// transforms' common 1/F^2 cancels); cross / den likewise
template <typename T>
__global__ void k_apm_crop(const T* __restrict__ num, const T* __restrict__ den, const T* __restrict__ cross,
                           int npix, int F, double* map, double* mcross) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)npix * npix) return;
  const int off = (npix - 1) / 2;
  const int i = (int)(t / npix), j = (int)(t % npix);
  const size_t o = (size_t)(i + off) * F + (j + off);
  const double d = (double)den[o];
  map[t] = (double)num[o] / d;
  if (cross && mcross) mcross[t] = (double)cross[o] / d;
}

// <Map^3> of every triplet i <= j <= k (extract_Map3_of_field :466-531): the
// mean over the window [c_k, npix - c_k)^2 of M_i M_j M_k, c_k the border of
// the triplet's largest aperture. One thread per pixel reads its n_theta map
// values once and, for each triplet whose window holds the pixel, adds the
// product to a per-block FP64 sum (warp shuffles, then one shared-memory
// atomic per warp); one global FP64 atomic per block and triplet.
constexpr int APM_MAX_THETA = 16;
constexpr int APM_MAX_TRIP = APM_MAX_THETA * (APM_MAX_THETA + 1) * (APM_MAX_THETA + 2) / 6;

__global__ void k_apm_map3(const double* __restrict__ maps, int npix, int n_theta, const int* __restrict__ cut,
                           double* sums) {
  __shared__ double s[APM_MAX_TRIP];
  const int ntrip = n_theta * (n_theta + 1) * (n_theta + 2) / 6;
  for (int q = threadIdx.x; q < ntrip; q += blockDim.x) s[q] = 0.0;
  __syncthreads();
  const long npx = (long)npix * npix;
  const long stride = (long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  // every thread of a warp runs the same number of iterations, so the
  // shuffles below always see the full warp
  const long iters = (npx + stride - 1) / stride;
  for (long it = 0; it < iters; ++it) {
    const long p = it * stride + (long)blockIdx.x * blockDim.x + threadIdx.x;
    double m[APM_MAX_THETA];
    int edge = -1;  // distance of the pixel to the nearest border
    if (p < npx) {
      const int i = (int)(p / npix), j = (int)(p % npix);
      edge = min(min(i, j), min(npix - 1 - i, npix - 1 - j));
      for (int a = 0; a < n_theta; ++a) m[a] = maps[(size_t)a * npx + p];
    } else {
      for (int a = 0; a < n_theta; ++a) m[a] = 0.0;
    }
    int q = 0;
    for (int a = 0; a < n_theta; ++a)
      for (int b = a; b < n_theta; ++b)
        for (int c = b; c < n_theta; ++c, ++q) {
          double v = (edge >= cut[c]) ? m[a] * m[b] * m[c] : 0.0;
          for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
          if (lane == 0 && v != 0.0) atomicAdd(&s[q], v);
        }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < ntrip; q += blockDim.x)
    if (s[q] != 0.0) atomicAdd(&sums[q], s[q]);
}

// The same sums for n_theta = NTH <= 5 apertures (up to 35 triplets): every
// thread keeps its triplets' partial sums in registers over its grid-stride
// pixels (one FP64 multiply per aperture pair and one FMA per triplet and
// pixel) and reduces them once at the end, instead of a warp reduction per
// triplet and pixel: about a fifth of the FP64 operations.
template <int NTH>
__global__ void k_apm_map3_reg(const double* __restrict__ maps, int npix, const int* __restrict__ cut, double* sums) {
  constexpr int NT3 = NTH * (NTH + 1) * (NTH + 2) / 6;
  __shared__ double s[NT3];
  for (int q = threadIdx.x; q < NT3; q += blockDim.x) s[q] = 0.0;
  int cutv[NTH];
#pragma unroll
  for (int a = 0; a < NTH; ++a) cutv[a] = cut[a];
  __syncthreads();
  double acc[NT3];
#pragma unroll
  for (int q = 0; q < NT3; ++q) acc[q] = 0.0;
  const long npx = (long)npix * npix;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += stride) {
    const int i = (int)(p / npix), j = (int)(p % npix);
    const int edge = min(min(i, j), min(npix - 1 - i, npix - 1 - j));
    double m[NTH];
#pragma unroll
    for (int a = 0; a < NTH; ++a) m[a] = maps[(size_t)a * npx + p];
    int q = 0;
#pragma unroll
    for (int a = 0; a < NTH; ++a)
#pragma unroll
      for (int b = a; b < NTH; ++b) {
        const double pab = m[a] * m[b];
#pragma unroll
        for (int c = b; c < NTH; ++c, ++q)
          if (edge >= cutv[c]) acc[q] = fma(pab, m[c], acc[q]);
      }
  }
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < NT3; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) atomicAdd(&s[q], v);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < NT3; q += blockDim.x) atomicAdd(&sums[q], s[q]);
}

__global__ void k_apm_means(const double* sums, const double* counts, int ntrip, double* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < ntrip) out[q] = sums[q] / counts[q];
}

unsigned blocks_for(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

// ---------------------------------------------------------------------------
struct tp_apm {
  tp_ctx* ctx = nullptr;  // must outlive the tp_apm's calls (not its destruction)
  int device = 0;
  int npix = 0, F = 0, n_theta = 0, polynomial = 0;
  int precision = TP_FP64;  // of the transforms and Fourier products
  size_t rsz = sizeof(double), csz = sizeof(double2);  // bytes of one real / complex transform value
  double fieldsize = 0;
  std::vector<double> thetas;
  std::string err;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  size_t nreal = 0, ncplx = 0;  // F*F, F*(F/2+1)
  // device state
  double* edges = nullptr;                          // [npix + 1]
  double *g_re = nullptr, *g_im = nullptr, *g_w = nullptr;  // CIC grids [npix][npix]
  // transform buffers, in the precision's real / complex type
  char* pad = nullptr;                              // [3][F][F] padded real grids
  char* spec = nullptr;                             // [3][F][F/2+1]: Re g, Im g, w
  char* qspec = nullptr;                            // [n_theta][3][F][F/2+1]: Re Q, Im Q, |Q|
  char* work = nullptr;                             // [3][F][F/2+1]: num, den, cross
  double* maps = nullptr;                           // [n_theta][npix][npix]
  double* mcross = nullptr;                         // [n_theta][npix][npix] (allocated on demand)
  char* uspec = nullptr;                            // [n_theta][F][F/2+1] U filter spectra (on demand)
  double* sums = nullptr;                           // [n_trip]
  double* counts = nullptr;                         // [n_trip]
  double* outv = nullptr;                           // [n_trip]
  int* cut = nullptr;                               // [n_theta]
  int* cut_same = nullptr;                          // [n_theta]
  std::vector<int> h_cut, h_cut_same;
  int n_trip() const { return n_theta * (n_theta + 1) * (n_theta + 2) / 6; }
  char* R(char* base, size_t q) const { return base + q * nreal * rsz; }  // q-th real grid
  char* Cx(char* base, size_t q) const { return base + q * ncplx * csz; }  // q-th spectrum
};

namespace {

int apm_fail(tp_apm* a, int st, const std::string& msg) {
  a->err = msg;
  if (a->ctx) tp_fail(a->ctx, st, msg);
  return st;
}
int apm_cuda(tp_apm* a, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return TP_OK;
  return apm_fail(a, TP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
int apm_fft(tp_apm* a, cufftResult r, const char* where) {
  if (r == CUFFT_SUCCESS) return TP_OK;
  return apm_fail(a, TP_ERR_CUDA, std::string(where) + ": cuFFT error " + std::to_string((int)r));
}

int fwd_fft(tp_apm* a, char* in, char* out) {
  const CufftApi& api = cufft();
  const cufftResult r = a->precision == TP_FP64
                            ? api.exec_d2z(a->fwd, (cufftDoubleReal*)in, (cufftDoubleComplex*)out)
                            : api.exec_r2c(a->fwd, (cufftReal*)in, (cufftComplex*)out);
  return apm_fft(a, r, "forward FFT");
}
int inv_fft(tp_apm* a, char* in, char* out) {
  const CufftApi& api = cufft();
  const cufftResult r = a->precision == TP_FP64
                            ? api.exec_z2d(a->inv, (cufftDoubleComplex*)in, (cufftDoubleReal*)out)
                            : api.exec_c2r(a->inv, (cufftComplex*)in, (cufftReal*)out);
  return apm_fft(a, r, "inverse FFT");
}

// border of extract_Map3_of_field (:492-503): int(round(theta / fieldsize *
// npix * f)), f = 4 for the exponential filter (99.8 % of its power inside
// 4 theta), 1 for the polynomial one; numpy rounds halves to even
int border(double theta, double fieldsize, int npix, int polynomial) {
  const double v = theta / fieldsize * npix * (polynomial ? 1.0 : 4.0);
  return (int)std::nearbyint(v);  // default rounding mode: to nearest, ties to even
}

// the per-field part: forward transforms of the three grids, then per
// aperture the products, two (three) inverse transforms and the crop; T / C
// the real / complex type of the transforms
template <typename T, typename C>
int apm_maps_t(tp_apm* a, bool want_cross) {
  cudaStream_t s = a->ctx->stream;
  const int n = a->npix, F = a->F;
  const long npx = (long)n * n;
  cudaError_t e = cudaMemsetAsync(a->pad, 0, a->rsz * 3 * a->nreal, s);
  if (e != cudaSuccess) return apm_cuda(a, e, "apm pad clear");
  const double* src[3] = {a->g_re, a->g_im, a->g_w};
  for (int q = 0; q < 3; ++q) k_apm_pad<T><<<blocks_for(npx, 256), 256, 0, s>>>(src[q], n, F, (T*)a->R(a->pad, q));
  e = cudaGetLastError();
  if (e != cudaSuccess) return apm_cuda(a, e, "apm pad");
  for (int q = 0; q < 3; ++q) {
    int st = fwd_fft(a, a->R(a->pad, q), a->Cx(a->spec, q));
    if (st) return st;
  }
  if (want_cross && !a->mcross) {
    e = cudaMalloc(&a->mcross, sizeof(double) * a->n_theta * npx);
    if (e != cudaSuccess) return apm_cuda(a, e, "apm cross maps");
  }
  const C* Y = (const C*)a->spec;
  for (int t = 0; t < a->n_theta; ++t) {
    const C* Q = (const C*)a->Cx(a->qspec, 3 * (size_t)t);
    C* W = (C*)a->work;
    const long nc = (long)a->ncplx;
    k_apm_spectra<C><<<blocks_for(nc, 256), 256, 0, s>>>(Y, Y + nc, Y + 2 * nc, Q, Q + nc, Q + 2 * nc, nc, W, W + nc,
                                                        want_cross ? W + 2 * nc : nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return apm_cuda(a, e, "apm spectra");
    for (int q = 0; q < (want_cross ? 3 : 2); ++q) {
      int st = inv_fft(a, a->Cx(a->work, q), a->R(a->pad, q));
      if (st) return st;
    }
    k_apm_crop<T><<<blocks_for(npx, 256), 256, 0, s>>>((const T*)a->R(a->pad, 0), (const T*)a->R(a->pad, 1),
                                                       want_cross ? (const T*)a->R(a->pad, 2) : nullptr, n, F,
                                                       a->maps + (size_t)t * npx,
                                                       want_cross ? a->mcross + (size_t)t * npx : nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return apm_cuda(a, e, "apm crop");
  }
  return TP_OK;
}

int apm_maps_device(tp_apm* a, bool want_cross) {
  return a->precision == TP_FP64 ? apm_maps_t<double, double2>(a, want_cross) : apm_maps_t<float, float2>(a, want_cross);
}

// the Fourier transforms of the Q filter grids of every aperture
template <typename T>
int apm_filters_t(tp_apm* a) {
  cudaStream_t s = a->ctx->stream;
  const long npx = (long)a->npix * a->npix;
  for (int t = 0; t < a->n_theta; ++t) {
    cudaError_t e = cudaMemsetAsync(a->pad, 0, a->rsz * 3 * a->nreal, s);
    if (e != cudaSuccess) return apm_cuda(a, e, "apm filter clear");
    k_apm_filter<T><<<blocks_for(npx, 256), 256, 0, s>>>(a->npix, a->F, a->fieldsize, a->thetas[t], a->polynomial,
                                                         (T*)a->R(a->pad, 0), (T*)a->R(a->pad, 1),
                                                         (T*)a->R(a->pad, 2));
    e = cudaGetLastError();
    if (e != cudaSuccess) return apm_cuda(a, e, "apm filter");
    for (int q = 0; q < 3; ++q) {
      int st = fwd_fft(a, a->R(a->pad, q), a->Cx(a->qspec, 3 * (size_t)t + q));
      if (st) return st;
    }
  }
  return apm_cuda(a, cudaStreamSynchronize(s), "apm filters");
}

int apm_map3_device(tp_apm* a, int same_fieldsize) {
  cudaStream_t s = a->ctx->stream;
  const int nt = a->n_trip();
  cudaError_t e = cudaMemsetAsync(a->sums, 0, sizeof(double) * nt, s);
  if (e != cudaSuccess) return apm_cuda(a, e, "apm sums");
  const int dev = a->ctx->device;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long npx = (long)a->npix * a->npix;
  unsigned grid = (unsigned)std::min<long>(blocks_for(npx, 256), (long)sms * 8);
  const int* cut = same_fieldsize ? a->cut_same : a->cut;
  switch (a->n_theta) {
    case 1: k_apm_map3_reg<1><<<grid, 256, 0, s>>>(a->maps, a->npix, cut, a->sums); break;
    case 2: k_apm_map3_reg<2><<<grid, 256, 0, s>>>(a->maps, a->npix, cut, a->sums); break;
    case 3: k_apm_map3_reg<3><<<grid, 256, 0, s>>>(a->maps, a->npix, cut, a->sums); break;
    case 4: k_apm_map3_reg<4><<<grid, 256, 0, s>>>(a->maps, a->npix, cut, a->sums); break;
    case 5: k_apm_map3_reg<5><<<grid, 256, 0, s>>>(a->maps, a->npix, cut, a->sums); break;
    default: k_apm_map3<<<grid, 256, 0, s>>>(a->maps, a->npix, a->n_theta, cut, a->sums);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return apm_cuda(a, e, "apm map3 launch");
  // pixel counts of the windows are known on the host
  std::vector<double> cnt(nt);
  const std::vector<int>& c = same_fieldsize ? a->h_cut_same : a->h_cut;
  int q = 0;
  for (int i = 0; i < a->n_theta; ++i)
    for (int j = i; j < a->n_theta; ++j)
      for (int k = j; k < a->n_theta; ++k, ++q) {
        const double side = a->npix - 2.0 * c[k];
        cnt[q] = side > 0 ? side * side : NAN;
      }
  e = cudaMemcpyAsync(a->counts, cnt.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_apm_means<<<blocks_for(nt, 128), 128, 0, s>>>(a->sums, a->counts, nt, a->outv);
    e = cudaGetLastError();
  }
  // the host vector must outlive the copy
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return apm_cuda(a, e, "apm map3");
}

int apm_grid_device(tp_apm* a, const double* x, const double* y, const double* g1, const double* g2, long n_gal) {
  cudaStream_t s = a->ctx->stream;
  const size_t g = sizeof(double) * a->npix * a->npix;
  cudaError_t e = cudaMemsetAsync(a->g_re, 0, g, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a->g_im, 0, g, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a->g_w, 0, g, s);
  if (e != cudaSuccess) return apm_cuda(a, e, "apm grid clear");
  if (n_gal > 0)
    k_apm_cic<<<blocks_for(n_gal, 256), 256, 0, s>>>(x, y, g1, g2, n_gal, a->edges, a->npix,
                                                     a->fieldsize / (a->npix - 1), a->g_re, a->g_im, a->g_w);
  return apm_cuda(a, cudaGetLastError(), "apm cic");
}

}  // namespace

extern "C" int tp_apm_destroy(tp_apm* a);

extern "C" int tp_apm_create(tp_ctx* ctx, int npix, double fieldsize, const double* thetas, int n_theta,
                             int polynomial, int precision, tp_apm** out) {
  TpRange nvtx_range("tp_apm_create");
  if (!ctx || !out || !thetas || npix < 8 || !(fieldsize > 0) || n_theta < 1 || n_theta > APM_MAX_THETA)
    return TP_ERR_ARG;
  if (precision != TP_FP64 && precision != TP_FP32) return TP_ERR_ARG;
  for (int i = 0; i < n_theta; ++i)
    if (!(thetas[i] > 0)) return tp_fail(ctx, TP_ERR_ARG, "aperture radii must be > 0");
  *out = nullptr;
  const CufftApi& api = cufft();
  if (!api.ok) return tp_fail(ctx, TP_ERR_STATE, api.why);
  cudaSetDevice(ctx->device);
  tp_apm* a = new tp_apm();
  a->ctx = ctx;
  a->device = ctx->device;
  a->npix = npix;
  a->fieldsize = fieldsize;
  a->n_theta = n_theta;
  a->polynomial = polynomial ? 1 : 0;
  a->precision = precision;
  a->rsz = precision == TP_FP64 ? sizeof(double) : sizeof(float);
  a->csz = precision == TP_FP64 ? sizeof(double2) : sizeof(float2);
  a->thetas.assign(thetas, thetas + n_theta);
  a->F = fft_size(2 * npix - 1);
  a->nreal = (size_t)a->F * a->F;
  a->ncplx = (size_t)a->F * (a->F / 2 + 1);
  const size_t npx = (size_t)npix * npix;
  const int nt = a->n_trip();
  auto fail = [&](int st) {
    tp_apm_destroy(a);
    return st;
  };
  cudaError_t e = cudaSuccess;
  auto M = [&](auto** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc((void**)p, bytes);
  };
  M(&a->edges, sizeof(double) * (npix + 1));
  M(&a->g_re, sizeof(double) * npx);
  M(&a->g_im, sizeof(double) * npx);
  M(&a->g_w, sizeof(double) * npx);
  M(&a->pad, a->rsz * 3 * a->nreal);
  M(&a->spec, a->csz * 3 * a->ncplx);
  M(&a->qspec, a->csz * 3 * a->ncplx * n_theta);
  M(&a->work, a->csz * 3 * a->ncplx);
  M(&a->maps, sizeof(double) * npx * n_theta);
  M(&a->sums, sizeof(double) * nt);
  M(&a->counts, sizeof(double) * nt);
  M(&a->outv, sizeof(double) * nt);
  M(&a->cut, sizeof(int) * n_theta);
  M(&a->cut_same, sizeof(int) * n_theta);
  if (e != cudaSuccess) return fail(tp_fail(ctx, TP_ERR_NOMEM, std::string("apm buffers: ") + cudaGetErrorString(e)));
  const bool f64 = precision == TP_FP64;
  if (api.plan2d(&a->fwd, a->F, a->F, f64 ? CUFFT_D2Z : CUFFT_R2C) != CUFFT_SUCCESS)
    return fail(tp_fail(ctx, TP_ERR_CUDA, "cufftPlan2d forward"));
  a->have_fwd = true;
  if (api.plan2d(&a->inv, a->F, a->F, f64 ? CUFFT_Z2D : CUFFT_C2R) != CUFFT_SUCCESS)
    return fail(tp_fail(ctx, TP_ERR_CUDA, "cufftPlan2d inverse"));
  a->have_inv = true;
  api.set_stream(a->fwd, ctx->stream);
  api.set_stream(a->inv, ctx->stream);
  // bin edges exactly as numpy forms them: arange(npix + 1) / (npix - 1) * fieldsize
  std::vector<double> edges(npix + 1);
  for (int i = 0; i <= npix; ++i) edges[i] = ((double)i / (double)(npix - 1)) * fieldsize;
  a->h_cut.resize(n_theta);
  a->h_cut_same.resize(n_theta);
  double tmax = 0;
  for (int i = 0; i < n_theta; ++i) tmax = std::max(tmax, thetas[i]);
  for (int i = 0; i < n_theta; ++i) {
    a->h_cut[i] = border(thetas[i], fieldsize, npix, a->polynomial);
    a->h_cut_same[i] = border(tmax, fieldsize, npix, a->polynomial);
  }
  cudaStream_t s = ctx->stream;
  e = cudaMemcpyAsync(a->edges, edges.data(), sizeof(double) * (npix + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->cut, a->h_cut.data(), sizeof(int) * n_theta, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(a->cut_same, a->h_cut_same.data(), sizeof(int) * n_theta, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(tp_cuda(ctx, e, "apm upload"));
  // the filter spectra of every aperture, computed once
  const int st = f64 ? apm_filters_t<double>(a) : apm_filters_t<float>(a);
  if (st) return fail(st);
  *out = a;
  return TP_OK;
}

extern "C" int tp_apm_destroy(tp_apm* a) {
  if (!a) return TP_OK;
  // only the device is used here: the context may already be gone
  cudaSetDevice(a->device);
  const CufftApi& api = cufft();
  if (a->have_fwd) api.destroy(a->fwd);
  if (a->have_inv) api.destroy(a->inv);
  for (void* p : {(void*)a->edges, (void*)a->g_re, (void*)a->g_im, (void*)a->g_w, (void*)a->pad, (void*)a->spec,
                  (void*)a->qspec, (void*)a->work, (void*)a->maps, (void*)a->mcross, (void*)a->sums, (void*)a->counts,
                  (void*)a->outv, (void*)a->cut, (void*)a->cut_same, (void*)a->uspec})
    if (p) cudaFree(p);
  delete a;
  return TP_OK;
}

extern "C" int tp_apm_fft_size(const tp_apm* a) { return a ? a->F : 0; }

extern "C" int tp_apm_grid(tp_apm* a, const double* x, const double* y, const double* g1, const double* g2,
                           long n_gal) {
  TpRange nvtx_range("tp_apm_grid");
  if (!a || n_gal < 0 || (n_gal > 0 && (!x || !y || !g1 || !g2))) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  const size_t b = sizeof(double) * (size_t)n_gal;
  const size_t o = (b + 255) & ~size_t(255);
  int st = a->ctx->ensure_io(4 * o + 256);
  if (st) return st;
  char* io = a->ctx->d_io;
  cudaStream_t s = a->ctx->stream;
  cudaError_t e = cudaSuccess;
  const double* h[4] = {x, y, g1, g2};
  for (int q = 0; q < 4 && e == cudaSuccess && n_gal > 0; ++q) e = cudaMemcpyAsync(io + q * o, h[q], b, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return apm_cuda(a, e, "apm catalogue upload");
  return apm_grid_device(a, (const double*)io, (const double*)(io + o), (const double*)(io + 2 * o),
                         (const double*)(io + 3 * o), n_gal);
}

extern "C" int tp_apm_grid_device(tp_apm* a, const double* x, const double* y, const double* g1, const double* g2,
                                  long n_gal) {
  if (!a || n_gal < 0 || (n_gal > 0 && (!x || !y || !g1 || !g2))) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  return apm_grid_device(a, x, y, g1, g2, n_gal);
}

extern "C" int tp_apm_set_grid(tp_apm* a, const double* shear_re, const double* shear_im, const double* weight) {
  if (!a || !shear_re || !shear_im || !weight) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  const size_t g = sizeof(double) * a->npix * a->npix;
  cudaStream_t s = a->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(a->g_re, shear_re, g, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->g_im, shear_im, g, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->g_w, weight, g, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return apm_cuda(a, e, "apm set grid");
}

extern "C" int tp_apm_get_grid(tp_apm* a, double* shear_re, double* shear_im, double* weight) {
  if (!a || !shear_re || !shear_im || !weight) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  const size_t g = sizeof(double) * a->npix * a->npix;
  cudaStream_t s = a->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(shear_re, a->g_re, g, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(shear_im, a->g_im, g, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(weight, a->g_w, g, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return apm_cuda(a, e, "apm get grid");
}

extern "C" int tp_apm_maps(tp_apm* a, double* maps, double* mcross) {
  TpRange nvtx_range("tp_apm_maps");
  if (!a) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  int st = apm_maps_device(a, mcross != nullptr);
  if (st) return st;
  const size_t b = sizeof(double) * a->npix * a->npix * a->n_theta;
  cudaStream_t s = a->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (maps) e = cudaMemcpyAsync(maps, a->maps, b, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && mcross) e = cudaMemcpyAsync(mcross, a->mcross, b, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return apm_cuda(a, e, "apm maps");
}

template <typename T, typename C>
int apm_kappa_t(tp_apm* a, const double* kappa) {
  cudaStream_t s = a->ctx->stream;
  const int n = a->npix, F = a->F;
  const long npx = (long)n * n;
  cudaError_t e = cudaSuccess;
  if (!a->uspec) {
    e = cudaMalloc(&a->uspec, a->csz * a->ncplx * a->n_theta);
    if (e != cudaSuccess) return apm_cuda(a, e, "apm U spectra");
    for (int t = 0; t < a->n_theta; ++t) {
      e = cudaMemsetAsync(a->pad, 0, a->rsz * a->nreal, s);
      if (e != cudaSuccess) return apm_cuda(a, e, "apm U filter clear");
      k_apm_ufilter<T><<<blocks_for(npx, 256), 256, 0, s>>>(n, F, a->fieldsize, a->thetas[t], (T*)a->pad);
      e = cudaGetLastError();
      if (e != cudaSuccess) return apm_cuda(a, e, "apm U filter");
      int st = fwd_fft(a, a->pad, a->Cx(a->uspec, t));
      if (st) return st;
    }
  }
  // the kappa grid goes through the shear grid's real-part buffer
  e = cudaMemcpyAsync(a->g_re, kappa, sizeof(double) * npx, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a->pad, 0, a->rsz * a->nreal, s);
  if (e != cudaSuccess) return apm_cuda(a, e, "apm kappa upload");
  k_apm_pad<T><<<blocks_for(npx, 256), 256, 0, s>>>(a->g_re, n, F, (T*)a->pad);
  int st = fwd_fft(a, a->pad, a->spec);
  if (st) return st;
  // Map_fft_from_kappa (:183-197): fftconvolve(kappa, U, 'same') * fieldsize^2 / npix^2;
  // the inverse transform is unnormalised (1 / F^2)
  const double scale = a->fieldsize * a->fieldsize / ((double)n * n) / ((double)F * F);
  for (int t = 0; t < a->n_theta; ++t) {
    k_apm_mul<C><<<blocks_for((long)a->ncplx, 256), 256, 0, s>>>((const C*)a->spec, (const C*)a->Cx(a->uspec, t),
                                                                (long)a->ncplx, (C*)a->work);
    st = inv_fft(a, a->work, a->R(a->pad, 1));
    if (st) return st;
    k_apm_crop_scaled<T><<<blocks_for(npx, 256), 256, 0, s>>>((const T*)a->R(a->pad, 1), n, F, scale,
                                                              a->maps + (size_t)t * npx);
  }
  return apm_cuda(a, cudaGetLastError(), "apm kappa maps");
}

extern "C" int tp_apm_maps_from_kappa(tp_apm* a, const double* kappa, double* maps) {
  TpRange nvtx_range("tp_apm_maps_from_kappa");
  if (!a || !kappa) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  int st = a->precision == TP_FP64 ? apm_kappa_t<double, double2>(a, kappa) : apm_kappa_t<float, float2>(a, kappa);
  if (st) return st;
  cudaStream_t s = a->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (maps)
    e = cudaMemcpyAsync(maps, a->maps, sizeof(double) * a->npix * a->npix * a->n_theta, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return apm_cuda(a, e, "apm kappa maps");
}

extern "C" int tp_apm_map3(tp_apm* a, int same_fieldsize, double* out) {
  TpRange nvtx_range("tp_apm_map3");
  if (!a || !out) return TP_ERR_ARG;
  cudaSetDevice(a->ctx->device);
  int st = apm_map3_device(a, same_fieldsize);
  if (st) return st;
  cudaError_t e = cudaMemcpy(out, a->outv, sizeof(double) * a->n_trip(), cudaMemcpyDeviceToHost);
  return apm_cuda(a, e, "apm map3 result");
}

extern "C" int tp_apm_extract_map3(tp_apm* a, const double* x, const double* y, const double* g1, const double* g2,
                                   long n_gal, int same_fieldsize, double* out) {
  TpRange nvtx_range("tp_apm_extract_map3");
  int st = tp_apm_grid(a, x, y, g1, g2, n_gal);
  if (st) return st;
  st = apm_maps_device(a, false);
  if (st) return st;
  return tp_apm_map3(a, same_fieldsize, out);
}

extern "C" int tp_apm_extract_map3_device(tp_apm* a, const double* x, const double* y, const double* g1,
                                          const double* g2, long n_gal, int same_fieldsize, double* out_device) {
  if (!a || !out_device) return TP_ERR_ARG;
  int st = tp_apm_grid_device(a, x, y, g1, g2, n_gal);
  if (st) return st;
  st = apm_maps_device(a, false);
  if (st) return st;
  st = apm_map3_device(a, same_fieldsize);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(out_device, a->outv, sizeof(double) * a->n_trip(), cudaMemcpyDeviceToDevice,
                                  a->ctx->stream);
  return apm_cuda(a, e, "apm map3 copy");
}
