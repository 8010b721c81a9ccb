// The b_kappa surrogate network on the 5th-generation tensor cores: a
// multilayer perceptron 8 -> 256 -> 256 -> 256 -> 256 -> 1 (SiLU after the
// hidden layers) trained and evaluated with BF16 operands and FP32
// accumulation. Every layer is one GEMM C = A B^T (A [M x K], B [N x K], both
// BF16 with K contiguous) on tcgen05: one CTA computes a 128 x N tile
// (N <= 256) into tensor memory, with K in 64-wide slabs staged in shared
// memory in the 128-byte-swizzled K-major layout (two buffers: the next slab
// loads while the tensor core consumes the current one); one thread issues
// the MMAs and commits them to the buffer's mbarrier; the four warps read the
// accumulator back (tcgen05.ld) and apply the layer's epilogue (bias, SiLU or
// its derivative, BF16 row-major and transposed copies for the next layer and
// the weight gradients, the last layer's dot product). Weight gradients are
// the same GEMM over the batch (K = batch) split into K slices whose FP32
// partials a second kernel sums in a fixed order.
//
// Every mbarrier wait has an iteration limit: on expiry the kernel raises an
// error flag, waits (bounded) for its committed MMAs, frees its tensor memory
// and skips the epilogue.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "tp_capi_internal.h"
#include "tp_kernels.cuh"

namespace tp {

constexpr int MLP_IN = 8;       // features
constexpr int MLP_IN_PAD = 64;  // first layer's K (one 64-wide slab, zero padded)
constexpr int MLP_W = 256;      // hidden width
constexpr int GEMM_NT = 128;    // threads of the GEMM CTA (4 warps = 128 TMEM lanes)
constexpr int GEMM_BM = 128;    // rows per CTA tile
constexpr int GEMM_BK = 64;     // K per slab (one 128-byte swizzle atom of BF16)
constexpr int MBAR_SPIN = 1 << 22;

enum GemmEpi : int {
  EPI_BIAS = 1,        // z += bias[col]
  EPI_DSILU = 2,       // z *= silu'(zin[row, col])
  EPI_STORE_Z = 4,     // zout[row, col] = z (FP32)
  EPI_SILU = 8,        // h = silu(z), else h = z
  EPI_STORE_H = 16,    // h_bf16[row, col]
  EPI_STORE_HT = 32,   // ht_bf16[col, row]
  EPI_STORE_F32 = 64,  // out_f32[split][row, col] = h
  EPI_DOT = 128,       // y[row] = sum_col h w5[col] + b5
};

struct GemmArgs {
  const __nv_bfloat16* A;
  int lda;
  const __nv_bfloat16* B;
  int ldb;
  int M, N, K;  // M % 128 == 0, N % 32 == 0 and 32 <= N <= 256, K % 64 == 0
  int kslices;  // grid.y; each CTA row covers K / kslices (a multiple of 64)
  int flags;
  const float* bias;
  const float* zin;
  int ldzin;
  float* zout;
  int ldz;
  __nv_bfloat16* h;
  int ldh;
  __nv_bfloat16* ht;
  int ldht;
  float* out;
  int ldo;
  long long split_stride;
  const float* w5;
  const float* b5;  // device scalar
  float* y;
  unsigned* err;  // bit 0: an mbarrier wait reached its limit
};

// ---- tcgen05 / mbarrier primitives (inline PTX) -----------------------------
__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity) {
  uint32_t ok = 0;
  for (int it = 0; it < MBAR_SPIN && !ok; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand tile in the 128-byte swizzle: rows of 64 BF16 (128 bytes),
// 8-row atoms of 1024 bytes (stride 1024), 1024-byte aligned base; the K
// step of 16 elements inside the atom advances the start address by 32 bytes
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}
// 32 consecutive accumulator columns of this warp's 32 lanes (one row per lane)
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%"
      "20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad_f(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// stage one 64-wide K slab of `rows` rows (K-major, 16-byte chunks) into the
// swizzled layout
__device__ __forceinline__ void load_slab(char* dst, const __nv_bfloat16* src, int ld, int rows, int k0) {
  const int chunks = rows * 8;
  for (int q = threadIdx.x; q < chunks; q += GEMM_NT) {
    const int r = q >> 3, c = q & 7;
    const uint4 v = *reinterpret_cast<const uint4*>(src + (size_t)r * ld + k0 + 8 * c);
    *reinterpret_cast<uint4*>(dst + r * 128 + ((c ^ (r & 7)) << 4)) = v;
  }
}

// dynamic shared memory: 2 x (A slab 16 KB + B slab up to 32 KB), 1024-aligned
constexpr size_t GEMM_SLAB_A = (size_t)GEMM_BM * GEMM_BK * 2;
constexpr size_t GEMM_SLAB_B = (size_t)MLP_W * GEMM_BK * 2;
constexpr size_t GEMM_SMEM = 1024 + 2 * (GEMM_SLAB_A + GEMM_SLAB_B) + 64;

__global__ void __launch_bounds__(GEMM_NT, 1) k_gemm_tc(GemmArgs g) {
  extern __shared__ __align__(16) char smem_raw[];
  // swizzled tiles need a 1024-byte aligned shared-memory address
  char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  char* sa[2] = {base, base + GEMM_SLAB_A};
  char* sb[2] = {base + 2 * GEMM_SLAB_A, base + 2 * GEMM_SLAB_A + GEMM_SLAB_B};
  uint64_t* bars = (uint64_t*)(base + 2 * (GEMM_SLAB_A + GEMM_SLAB_B));
  uint32_t* s_tmem = (uint32_t*)(bars + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * GEMM_BM;
  const int kper = g.K / g.kslices, kbeg = blockIdx.y * kper;
  const int nslab = kper / GEMM_BK;
  const int N = g.N;
  const int ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]);

  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_tmem;
  const uint32_t idesc = idesc_bf16_m128(N);
  bool ok = true;

  for (int s = 0; s < nslab && ok; ++s) {
    const int b = s & 1;
    if (s >= 2) ok = mbar_wait(b ? bar1 : bar0, ((s - 2) >> 1) & 1);  // buffer b free again
    ok = __syncthreads_and(ok);
    if (!ok) break;
    const int k0 = kbeg + s * GEMM_BK;
    load_slab(sa[b], g.A + (size_t)m0 * g.lda, g.lda, GEMM_BM, k0);
    load_slab(sb[b], g.B, g.ldb, N, k0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sa[b]), b0 = smem_u32(sb[b]);
#pragma unroll
      for (int kk = 0; kk < GEMM_BK / 16; ++kk)
        tc_mma(tmem, smem_desc_sw128(a0 + 32 * kk), smem_desc_sw128(b0 + 32 * kk), idesc, (s | kk) != 0);
      tc_commit(b ? bar1 : bar0);
    }
  }
  // the last commit covers every MMA of the CTA
  if (nslab > 0) {
    const int last = nslab - 1;
    const bool done = mbar_wait((last & 1) ? bar1 : bar0, (last >> 1) & 1);
    ok = ok && done;
  }
  ok = __syncthreads_and(ok);
  tc_fence_after();

  if (ok && nslab > 0) {
    const int row0 = m0 + warp * 32;  // this warp's 32 rows; lane = row in the accumulator
    const int row = row0 + lane;
    const uint32_t tw = tmem + ((uint32_t)(warp * 32) << 16);
    float dot = 0.f;
    const int f = g.flags;
    // Row-major operands and results go through a per-warp 32 x 33 shared
    // tile (the slab buffers are free once the last MMA has completed), so
    // that global loads and stores move whole rows (32 consecutive columns per
    // instruction) instead of one element per lane and row.
    float* tile = reinterpret_cast<float*>(sb[0]) + warp * 32 * 33;
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tc_ld32(tw + (uint32_t)c0, v);
      float zin[32];
      if (f & EPI_DSILU) {
        for (int r = 0; r < 32; ++r) tile[r * 33 + lane] = g.zin[(size_t)(row0 + r) * g.ldzin + c0 + lane];
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j) zin[j] = tile[lane * 33 + j];
        __syncwarp();
      }
      float zv[32], hv[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = c0 + j;
        float z = v[j];
        if (f & EPI_BIAS) z += g.bias[col];
        if (f & EPI_DSILU) z *= silu_grad_f(zin[j]);
        zv[j] = z;
        const float hval = (f & EPI_SILU) ? silu_f(z) : z;
        hv[j] = hval;
        if (f & EPI_STORE_HT) g.ht[(size_t)col * g.ldht + row] = __float2bfloat16_rn(hval);
        if (f & EPI_DOT) dot = fmaf(hval, g.w5[col], dot);
      }
      if (f & EPI_STORE_Z) {
#pragma unroll
        for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = zv[j];
        __syncwarp();
        for (int r = 0; r < 32; ++r) g.zout[(size_t)(row0 + r) * g.ldz + c0 + lane] = tile[r * 33 + lane];
        __syncwarp();
      }
      if (f & (EPI_STORE_F32 | EPI_STORE_H)) {
#pragma unroll
        for (int j = 0; j < 32; ++j) tile[lane * 33 + j] = hv[j];
        __syncwarp();
        for (int r = 0; r < 32; ++r) {
          const float x = tile[r * 33 + lane];
          if (f & EPI_STORE_F32)
            g.out[(size_t)blockIdx.y * g.split_stride + (size_t)(row0 + r) * g.ldo + c0 + lane] = x;
          if (f & EPI_STORE_H) g.h[(size_t)(row0 + r) * g.ldh + c0 + lane] = __float2bfloat16_rn(x);
        }
        __syncwarp();
      }
    }
    if (f & EPI_DOT) g.y[row] = dot + *g.b5;
  }
  if (!ok && threadIdx.x == 0 && g.err) atomicOr(g.err, 1u);
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// ---- element-wise and reduction kernels of the training step ---------------

// features [n][8] (FP32) -> X [Mpad][64] and XT [64][Mpad] (BF16, zero padded)
__global__ void k_mlp_pack(const float* x, long n, int mpad, __nv_bfloat16* X, __nv_bfloat16* XT) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)mpad * MLP_IN_PAD) return;
  const int r = (int)(i / MLP_IN_PAD), c = (int)(i % MLP_IN_PAD);
  const float v = (r < n && c < MLP_IN) ? x[(size_t)r * MLP_IN + c] : 0.f;
  X[i] = __float2bfloat16_rn(v);
  XT[(size_t)c * mpad + r] = __float2bfloat16_rn(v);
}

// dy = 2 (y - t) / n (0 on padding rows); per-block partial sums of (y - t)^2
__global__ void k_mlp_loss(const float* y, const float* t, long n, int mpad, float* dy, double* part) {
  __shared__ double red[256];
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double e2 = 0;
  if (i < mpad) {
    float d = 0.f;
    if (i < n) {
      d = y[i] - t[i];
      e2 = (double)d * d;
    }
    dy[i] = i < n ? 2.f * d / (float)n : 0.f;
  }
  red[threadIdx.x] = e2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// sum of nparts doubles in a fixed order (one thread)
__global__ void k_sum_fixed(const double* part, int nparts, long n, float* loss) {
  if (threadIdx.x || blockIdx.x) return;
  double s = 0;
  for (int i = 0; i < nparts; ++i) s += part[i];
  *loss = (float)(s / (double)n);
}

// dW5[j] = sum_b dy[b] h4[b][j], db5 = sum_b dy[b]: one warp per column j
// (and one extra warp for db5), fixed summation order per lane then butterfly
__global__ void k_mlp_last_grad(const float* dy, const float* h4, int mpad, float* gw5, float* gb5) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w > MLP_W) return;
  float s = 0.f;
  for (int b = lane; b < mpad; b += 32) s += dy[b] * (w < MLP_W ? h4[(size_t)b * MLP_W + w] : 1.f);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    if (w < MLP_W)
      gw5[w] = s;
    else
      *gb5 = s;
  }
}

// dZ4 = dy w5 silu'(Z4): row-major and transposed BF16
__global__ void k_mlp_dz4(const float* dy, const float* w5, const float* z4, int mpad, __nv_bfloat16* dz,
                          __nv_bfloat16* dzt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long)mpad * MLP_W) return;
  const int r = (int)(i / MLP_W), c = (int)(i % MLP_W);
  const float v = dy[r] * w5[c] * silu_grad_f(z4[i]);
  dz[i] = __float2bfloat16_rn(v);
  dzt[(size_t)c * mpad + r] = __float2bfloat16_rn(v);
}

// bias gradient: db[j] = sum_b dZ[b][j] from the transposed copy (row j
// contiguous over the batch); one warp per j
__global__ void k_mlp_rowsum(const __nv_bfloat16* dzt, int rows, int mpad, float* db) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= rows) return;
  float s = 0.f;
  for (int b = lane; b < mpad; b += 32) s += __bfloat162float(dzt[(size_t)w * mpad + b]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) db[w] = s;
}

// out[i] = sum_s part[s][i] in a fixed order
__global__ void k_split_reduce(const float* part, int slices, long count, long stride, float* out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = 0.f;
  for (int k = 0; k < slices; ++k) s += part[(size_t)k * stride + i];
  out[i] = s;
}

// Adam (Kingma & Ba 2015, bias-corrected) on the FP32 master copy, then the
// BF16 copies the GEMMs read: w_bf [rows][ld_bf] and optionally its transpose
// wt_bf [cols][rows]; cols <= ld_bf, the padding columns stay zero
__global__ void k_mlp_adam(float* w, const float* g, float* m, float* v, long count, int cols, float lr, float b1,
                           float b2, float eps, float c1, float c2, __nv_bfloat16* w_bf, int ld_bf,
                           __nv_bfloat16* wt_bf, int rows) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (w_bf) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    w_bf[(size_t)r * ld_bf + c] = __float2bfloat16_rn(wi);
    if (wt_bf) wt_bf[(size_t)c * rows + r] = __float2bfloat16_rn(wi);
  }
}

// BF16 copies of an FP32 weight matrix (after set_params)
__global__ void k_mlp_cast(const float* w, long count, int cols, __nv_bfloat16* w_bf, int ld_bf, __nv_bfloat16* wt_bf,
                           int rows) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int r = (int)(i / cols), c = (int)(i % cols);
  w_bf[(size_t)r * ld_bf + c] = __float2bfloat16_rn(w[i]);
  if (wt_bf) wt_bf[(size_t)c * rows + r] = __float2bfloat16_rn(w[i]);
}

}  // namespace tp

// ---------------------------------------------------------------------------
// host side: the network's device state and its C ABI
// ---------------------------------------------------------------------------
using namespace tp;

namespace {

// FP32 master parameters and Adam moments, flat: W1 [256][8], b1, W2..W4
// [256][256], b2..b4, W5 [1][256], b5 (the host API's FP64 layout)
constexpr long P_W1 = 0, P_B1 = P_W1 + (long)MLP_W * MLP_IN;
constexpr long P_W2 = P_B1 + MLP_W, P_B2 = P_W2 + (long)MLP_W * MLP_W;
constexpr long P_W3 = P_B2 + MLP_W, P_B3 = P_W3 + (long)MLP_W * MLP_W;
constexpr long P_W4 = P_B3 + MLP_W, P_B4 = P_W4 + (long)MLP_W * MLP_W;
constexpr long P_W5 = P_B4 + MLP_W, P_B5 = P_W5 + MLP_W;
constexpr long P_COUNT = P_B5 + 1;
const long P_W[5] = {P_W1, P_W2, P_W3, P_W4, P_W5};
const long P_B[5] = {P_B1, P_B2, P_B3, P_B4, P_B5};
const int L_IN[5] = {MLP_IN, MLP_W, MLP_W, MLP_W, MLP_W};
const int L_OUT[5] = {MLP_W, MLP_W, MLP_W, MLP_W, 1};

int round_up(long n, int m) { return (int)((n + m - 1) / m * m); }

}  // namespace

struct tp_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  int max_rows = 0;  // padded batch capacity (multiple of 128)
  int kslices_max = 1;
  long adam_t = 0;
  std::string err;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // [P_COUNT]
  __nv_bfloat16* wb[4] = {};  // W1 [256][64] (padded), W2..W4 [256][256]
  __nv_bfloat16* wt[4] = {};  // transposes of W2..W4 (index 1..3; [0] unused)
  __nv_bfloat16 *X = nullptr, *XT = nullptr;
  float* Z[4] = {};
  __nv_bfloat16* H[3] = {};
  __nv_bfloat16* HT[3] = {};
  float* H4 = nullptr;
  float *y = nullptr, *t = nullptr, *dy = nullptr, *xin = nullptr;
  __nv_bfloat16* dZ[2] = {};
  __nv_bfloat16* dZT[2] = {};
  float* split = nullptr;  // [kslices][256][256]
  double* lpart = nullptr;
  float* loss = nullptr;
  unsigned* d_err = nullptr;
};

static int mlp_fail(tp_mlp* m, int st, const std::string& msg) {
  if (m) m->err = msg;
  return st;
}
static int mlp_cuda(tp_mlp* m, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return TP_OK;
  return mlp_fail(m, TP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

template <class T>
static cudaError_t dmalloc(T** p, size_t count) {
  return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

static cudaError_t gemm(tp_mlp* m, GemmArgs a) {
  static thread_local int attr_dev = -1;
  if (attr_dev != m->device) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM);
    if (e != cudaSuccess) return e;
    attr_dev = m->device;
  }
  if (a.M % GEMM_BM || a.N % 32 || a.N < 32 || a.N > MLP_W || a.K % GEMM_BK || a.kslices < 1 ||
      (a.K / a.kslices) % GEMM_BK || a.K % a.kslices)
    return cudaErrorInvalidValue;
  a.err = m->d_err;
  k_gemm_tc<<<dim3(a.M / GEMM_BM, a.kslices), GEMM_NT, GEMM_SMEM, m->stream>>>(a);
  return cudaGetLastError();
}

static GemmArgs gemm_args(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K) {
  GemmArgs a{};
  a.A = A;
  a.lda = lda;
  a.B = B;
  a.ldb = ldb;
  a.M = M;
  a.N = N;
  a.K = K;
  a.kslices = 1;
  return a;
}

// BF16 copies of the weights from the FP32 masters
static cudaError_t mlp_cast_all(tp_mlp* m) {
  for (int l = 0; l < 4; ++l) {
    const long cnt = (long)L_OUT[l] * L_IN[l];
    k_mlp_cast<<<(unsigned)((cnt + 255) / 256), 256, 0, m->stream>>>(
        m->p + P_W[l], cnt, L_IN[l], m->wb[l], l == 0 ? MLP_IN_PAD : MLP_W, l == 0 ? nullptr : m->wt[l], MLP_W);
  }
  return cudaGetLastError();
}

// forward over `rows` (multiple of 128) packed rows; training also keeps the
// pre-activations and transposed activations for the backward pass
static cudaError_t mlp_forward_dev(tp_mlp* m, int rows, bool train) {
  cudaError_t e = cudaSuccess;
  const __nv_bfloat16* a = m->X;
  int lda = MLP_IN_PAD;
  for (int l = 0; l < 4 && e == cudaSuccess; ++l) {
    GemmArgs g = gemm_args(a, lda, m->wb[l], l == 0 ? MLP_IN_PAD : MLP_W, rows, MLP_W, l == 0 ? MLP_IN_PAD : MLP_W);
    g.bias = m->p + P_B[l];
    g.flags = EPI_BIAS | EPI_SILU;
    if (train) {
      g.flags |= EPI_STORE_Z;
      g.zout = m->Z[l];
      g.ldz = MLP_W;
    }
    if (l < 3) {
      g.flags |= EPI_STORE_H;
      g.h = m->H[l];
      g.ldh = MLP_W;
      if (train) {
        g.flags |= EPI_STORE_HT;
        g.ht = m->HT[l];
        g.ldht = rows;
      }
    } else {
      g.flags |= EPI_DOT;
      g.w5 = m->p + P_W5;
      g.b5 = m->p + P_B5;
      g.y = m->y;
      if (train) {
        g.flags |= EPI_STORE_F32;
        g.out = m->H4;
        g.ldo = MLP_W;
      }
    }
    e = gemm(m, g);
    a = m->H[l < 3 ? l : 0];
    lda = MLP_W;
  }
  return e;
}

static int mlp_check(tp_mlp* m) {
  unsigned h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, m->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return mlp_cuda(m, e, "mlp");
  if (h) {
    cudaMemsetAsync(m->d_err, 0, sizeof(unsigned), m->stream);
    return mlp_fail(m, TP_ERR_CUDA, "mlp: a tensor-core wait reached its iteration limit");
  }
  return TP_OK;
}

// gradients of the mean squared error into m->g (forward included)
static cudaError_t mlp_backward_dev(tp_mlp* m, long n, int rows) {
  cudaError_t e = cudaSuccess;
  const int nb = (rows + 255) / 256;
  k_mlp_loss<<<nb, 256, 0, m->stream>>>(m->y, m->t, n, rows, m->dy, m->lpart);
  k_sum_fixed<<<1, 32, 0, m->stream>>>(m->lpart, nb, n, m->loss);
  k_mlp_last_grad<<<(MLP_W + 1 + 7) / 8, 256, 0, m->stream>>>(m->dy, m->H4, rows, m->g + P_W5, m->g + P_B5);
  k_mlp_dz4<<<(unsigned)(((long)rows * MLP_W + 255) / 256), 256, 0, m->stream>>>(m->dy, m->p + P_W5, m->Z[3], rows,
                                                                                 m->dZ[0], m->dZT[0]);
  e = cudaGetLastError();
  // K slices of the weight-gradient GEMMs: 1024 batch rows each (at most the
  // allocated partial buffers)
  int ks = rows / 1024;
  if (ks < 1) ks = 1;
  while (ks > m->kslices_max || rows % ks || (rows / ks) % GEMM_BK) --ks;
  int cur = 0;
  for (int l = 3; l >= 0 && e == cudaSuccess; --l) {
    const int in = l == 0 ? MLP_IN_PAD : MLP_W;
    // dW_l = dZ_l^T H_{l-1}: A = dZT [256][rows], B = H_{l-1}^T [in][rows]
    GemmArgs g = gemm_args(m->dZT[cur], rows, l == 0 ? m->XT : m->HT[l - 1], rows, MLP_W, in, rows);
    g.kslices = ks;
    g.flags = EPI_STORE_F32;
    g.out = ks > 1 ? m->split : m->g + P_W[l];
    g.ldo = in;
    g.split_stride = (long long)MLP_W * in;
    if (l == 0) {  // W1's gradient has 8 real columns of the 64 computed
      g.out = m->split;
    }
    e = gemm(m, g);
    if (e != cudaSuccess) break;
    if (l == 0) {
      // sum the slices into [256][64], then keep the 8 real columns
      k_split_reduce<<<(unsigned)(((long)MLP_W * in + 255) / 256), 256, 0, m->stream>>>(
          m->split, ks, (long)MLP_W * in, (long)MLP_W * in, m->split + (size_t)ks * MLP_W * in);
      e = cudaMemcpy2DAsync(m->g + P_W1, sizeof(float) * MLP_IN, m->split + (size_t)ks * MLP_W * in,
                            sizeof(float) * in, sizeof(float) * MLP_IN, MLP_W, cudaMemcpyDeviceToDevice, m->stream);
    } else if (ks > 1) {
      k_split_reduce<<<(unsigned)(((long)MLP_W * in + 255) / 256), 256, 0, m->stream>>>(
          m->split, ks, (long)MLP_W * in, (long)MLP_W * in, m->g + P_W[l]);
    }
    k_mlp_rowsum<<<MLP_W / 8, 256, 0, m->stream>>>(m->dZT[cur], MLP_W, rows, m->g + P_B[l]);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (l == 0 || e != cudaSuccess) break;
    // dZ_{l-1} = (dZ_l W_l) * silu'(Z_{l-1}): B = W_l^T [in][out]
    GemmArgs d = gemm_args(m->dZ[cur], MLP_W, m->wt[l], MLP_W, rows, MLP_W, MLP_W);
    d.flags = EPI_DSILU | EPI_STORE_H | EPI_STORE_HT;
    d.zin = m->Z[l - 1];
    d.ldzin = MLP_W;
    d.h = m->dZ[cur ^ 1];
    d.ldh = MLP_W;
    d.ht = m->dZT[cur ^ 1];
    d.ldht = rows;
    e = gemm(m, d);
    cur ^= 1;
  }
  return e;
}

static cudaError_t mlp_adam_dev(tp_mlp* m, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  m->adam_t++;
  const float c1 = 1.f - powf(b1, (float)m->adam_t), c2 = 1.f - powf(b2, (float)m->adam_t);
  for (int l = 0; l < 5; ++l) {
    const long cw = (long)L_OUT[l] * L_IN[l];
    __nv_bfloat16* wb = l < 4 ? m->wb[l] : nullptr;
    __nv_bfloat16* wt = (l >= 1 && l < 4) ? m->wt[l] : nullptr;
    k_mlp_adam<<<(unsigned)((cw + 255) / 256), 256, 0, m->stream>>>(
        m->p + P_W[l], m->g + P_W[l], m->m + P_W[l], m->v + P_W[l], cw, L_IN[l], lr, b1, b2, eps, c1, c2, wb,
        l == 0 ? MLP_IN_PAD : MLP_W, wt, MLP_W);
    const long cb = L_OUT[l];
    k_mlp_adam<<<(unsigned)((cb + 255) / 256), 256, 0, m->stream>>>(
        m->p + P_B[l], m->g + P_B[l], m->m + P_B[l], m->v + P_B[l], cb, 1, lr, b1, b2, eps, c1, c2, nullptr, 0,
        nullptr, 0);
  }
  return cudaGetLastError();
}

static cudaError_t mlp_upload_x(tp_mlp* m, const double* x, long n, int rows) {
  std::vector<float> xf((size_t)n * MLP_IN);
  for (size_t i = 0; i < xf.size(); ++i) xf[i] = (float)x[i];
  cudaError_t e = cudaMemcpyAsync(m->xin, xf.data(), sizeof(float) * xf.size(), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);  // xf leaves scope
  if (e == cudaSuccess) {
    k_mlp_pack<<<(unsigned)(((long)rows * MLP_IN_PAD + 255) / 256), 256, 0, m->stream>>>(m->xin, n, rows, m->X,
                                                                                           m->XT);
    e = cudaGetLastError();
  }
  return e;
}

extern "C" long tp_mlp_param_count(void) { return P_COUNT; }

extern "C" void tp_mlp_destroy(tp_mlp* m);

extern "C" int tp_mlp_create(int device, int max_batch, tp_mlp** out) {
  if (!out || max_batch < 1 || max_batch > (1 << 22)) return TP_ERR_ARG;
  *out = nullptr;
  tp_mlp* m = new tp_mlp();
  m->device = device;
  m->max_rows = round_up(max_batch, 1024);
  m->kslices_max = m->max_rows / 1024;
  const size_t R = (size_t)m->max_rows;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  for (float** q : {&m->p, &m->g, &m->m, &m->v})
    if (e == cudaSuccess) e = dmalloc(q, P_COUNT);
  if (e == cudaSuccess) e = dmalloc(&m->wb[0], (size_t)MLP_W * MLP_IN_PAD);
  for (int l = 1; l < 4; ++l) {
    if (e == cudaSuccess) e = dmalloc(&m->wb[l], (size_t)MLP_W * MLP_W);
    if (e == cudaSuccess) e = dmalloc(&m->wt[l], (size_t)MLP_W * MLP_W);
  }
  if (e == cudaSuccess) e = dmalloc(&m->X, R * MLP_IN_PAD);
  if (e == cudaSuccess) e = dmalloc(&m->XT, R * MLP_IN_PAD);
  for (int l = 0; l < 4; ++l)
    if (e == cudaSuccess) e = dmalloc(&m->Z[l], R * MLP_W);
  for (int l = 0; l < 3; ++l) {
    if (e == cudaSuccess) e = dmalloc(&m->H[l], R * MLP_W);
    if (e == cudaSuccess) e = dmalloc(&m->HT[l], R * MLP_W);
  }
  if (e == cudaSuccess) e = dmalloc(&m->H4, R * MLP_W);
  for (float** q : {&m->y, &m->t, &m->dy})
    if (e == cudaSuccess) e = dmalloc(q, R);
  if (e == cudaSuccess) e = dmalloc(&m->xin, R * MLP_IN);
  for (int i = 0; i < 2; ++i) {
    if (e == cudaSuccess) e = dmalloc(&m->dZ[i], R * MLP_W);
    if (e == cudaSuccess) e = dmalloc(&m->dZT[i], R * MLP_W);
  }
  if (e == cudaSuccess) e = dmalloc(&m->split, (size_t)(m->kslices_max + 1) * MLP_W * MLP_W);
  if (e == cudaSuccess) e = dmalloc(&m->lpart, R / 256 + 1);
  if (e == cudaSuccess) e = dmalloc(&m->loss, 1);
  if (e == cudaSuccess) e = dmalloc(&m->d_err, 1);
  // zero everything the padding relies on (padded weight columns, moments)
  if (e == cudaSuccess) e = cudaMemsetAsync(m->wb[0], 0, sizeof(__nv_bfloat16) * MLP_W * MLP_IN_PAD, m->stream);
  for (float* q : {m->p, m->g, m->m, m->v})
    if (e == cudaSuccess) e = cudaMemsetAsync(q, 0, sizeof(float) * P_COUNT, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_err, 0, sizeof(unsigned), m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    tp_mlp_destroy(m);
    return TP_ERR_CUDA;
  }
  *out = m;
  return TP_OK;
}

extern "C" void tp_mlp_destroy(tp_mlp* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  for (void* q : {(void*)m->p, (void*)m->g, (void*)m->m, (void*)m->v, (void*)m->X, (void*)m->XT, (void*)m->H4,
                  (void*)m->y, (void*)m->t, (void*)m->dy, (void*)m->xin, (void*)m->split, (void*)m->lpart,
                  (void*)m->loss, (void*)m->d_err})
    cudaFree(q);
  for (int l = 0; l < 4; ++l) {
    cudaFree(m->wb[l]);
    cudaFree(m->wt[l]);
    cudaFree(m->Z[l]);
  }
  for (int l = 0; l < 3; ++l) {
    cudaFree(m->H[l]);
    cudaFree(m->HT[l]);
  }
  for (int i = 0; i < 2; ++i) {
    cudaFree(m->dZ[i]);
    cudaFree(m->dZT[i]);
  }
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

extern "C" const char* tp_mlp_last_error(const tp_mlp* m) { return m ? m->err.c_str() : ""; }

extern "C" int tp_mlp_set_params(tp_mlp* m, const double* params) {
  if (!m || !params) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  std::vector<float> f(P_COUNT);
  for (long i = 0; i < P_COUNT; ++i) f[i] = (float)params[i];
  cudaError_t e = cudaMemcpyAsync(m->p, f.data(), sizeof(float) * P_COUNT, cudaMemcpyHostToDevice, m->stream);
  for (float* q : {m->m, m->v})
    if (e == cudaSuccess) e = cudaMemsetAsync(q, 0, sizeof(float) * P_COUNT, m->stream);
  if (e == cudaSuccess) e = mlp_cast_all(m);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  m->adam_t = 0;
  return mlp_cuda(m, e, "mlp set_params");
}

extern "C" int tp_mlp_get_params(tp_mlp* m, double* params) {
  if (!m || !params) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  std::vector<float> f(P_COUNT);
  cudaError_t e = cudaMemcpyAsync(f.data(), m->p, sizeof(float) * P_COUNT, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) return mlp_cuda(m, e, "mlp get_params");
  for (long i = 0; i < P_COUNT; ++i) params[i] = f[i];
  return TP_OK;
}

// y[n] for features x[n][8] (host buffers), in batches of the capacity
extern "C" int tp_mlp_forward(tp_mlp* m, const double* x, long n, double* y) {
  if (!m || !x || !y || n < 0) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  std::vector<float> yf;
  for (long s = 0; s < n; s += m->max_rows) {
    const long c = n - s < m->max_rows ? n - s : m->max_rows;
    const int rows = round_up(c, GEMM_BM);
    cudaError_t e = mlp_upload_x(m, x + s * MLP_IN, c, rows);
    if (e == cudaSuccess) e = mlp_forward_dev(m, rows, false);
    if (e != cudaSuccess) return mlp_cuda(m, e, "mlp forward");
    yf.resize(c);
    e = cudaMemcpyAsync(yf.data(), m->y, sizeof(float) * c, cudaMemcpyDeviceToHost, m->stream);
    if (e != cudaSuccess) return mlp_cuda(m, e, "mlp forward");
    const int st = mlp_check(m);
    if (st) return st;
    for (long i = 0; i < c; ++i) y[s + i] = yf[i];
  }
  return TP_OK;
}

// loss and gradients (flat FP64, the parameter layout) of the mean squared
// error on one batch, without an update
extern "C" int tp_mlp_gradients(tp_mlp* m, const double* x, const double* t, long n, double* grads, double* loss) {
  if (!m || !x || !t || n < 1 || n > m->max_rows) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  const int rows = round_up(n, GEMM_BM);
  cudaError_t e = mlp_upload_x(m, x, n, rows);
  std::vector<float> tf(n);
  for (long i = 0; i < n; ++i) tf[i] = (float)t[i];
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->t, tf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = mlp_forward_dev(m, rows, true);
  if (e == cudaSuccess) e = mlp_backward_dev(m, n, rows);
  std::vector<float> gf(P_COUNT);
  float lf = 0.f;
  if (e == cudaSuccess) e = cudaMemcpyAsync(gf.data(), m->g, sizeof(float) * P_COUNT, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&lf, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e != cudaSuccess) return mlp_cuda(m, e, "mlp gradients");
  const int st = mlp_check(m);
  if (st) return st;
  if (grads)
    for (long i = 0; i < P_COUNT; ++i) grads[i] = gf[i];
  if (loss) *loss = lf;
  return TP_OK;
}

// one Adam step on one batch given in device memory (x [n][8], t [n], FP32),
// asynchronous on the network's stream; *loss_dev receives the batch's loss
extern "C" int tp_mlp_train_step_device(tp_mlp* m, const float* x_dev, const float* t_dev, long n, float lr,
                                        float* loss_dev) {
  if (!m || !x_dev || !t_dev || n < 1 || n > m->max_rows) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  const int rows = round_up(n, GEMM_BM);
  cudaError_t e = cudaMemcpyAsync(m->xin, x_dev, sizeof(float) * n * MLP_IN, cudaMemcpyDeviceToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->t, t_dev, sizeof(float) * n, cudaMemcpyDeviceToDevice, m->stream);
  if (e == cudaSuccess) {
    k_mlp_pack<<<(unsigned)(((long)rows * MLP_IN_PAD + 255) / 256), 256, 0, m->stream>>>(m->xin, n, rows, m->X,
                                                                                           m->XT);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = mlp_forward_dev(m, rows, true);
  if (e == cudaSuccess) e = mlp_backward_dev(m, n, rows);
  if (e == cudaSuccess) e = mlp_adam_dev(m, lr);
  if (e == cudaSuccess && loss_dev)
    e = cudaMemcpyAsync(loss_dev, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, m->stream);
  return mlp_cuda(m, e, "mlp train step");
}

// status of the asynchronous steps so far (synchronises the stream)
extern "C" int tp_mlp_sync(tp_mlp* m) {
  if (!m) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  return mlp_check(m);
}

extern "C" void* tp_mlp_stream(const tp_mlp* m) { return m ? (void*)m->stream : nullptr; }

// C = A B^T (BF16 operands with K contiguous, FP32 result, device pointers) on
// the network's stream: M % 128 == 0, N % 32 == 0 with 32 <= N <= 256,
// K % 64 == 0; the tensor-core GEMM every layer uses
extern "C" int tp_gemm_bf16_device(tp_mlp* m, const void* A, int lda, const void* B, int ldb, float* C, int ldc,
                                   int M, int N, int K) {
  if (!m || !A || !B || !C || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N) return TP_ERR_ARG;
  cudaSetDevice(m->device);
  GemmArgs g = gemm_args((const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)B, ldb, M, N, K);
  g.flags = EPI_STORE_F32;
  g.out = C;
  g.ldo = ldc;
  cudaError_t e = gemm(m, g);
  if (e == cudaErrorInvalidValue) return mlp_fail(m, TP_ERR_ARG, "gemm: unsupported shape");
  if (e != cudaSuccess) return mlp_cuda(m, e, "gemm");
  return mlp_check(m);
}
