// BiHalofit bispectrum (Takahashi et al. 2020, Eqs. B4-B9) evaluated at one
// fixed line-of-sight node from precomputed per-node coefficients; the same
// formula as the reference's bispec (cuda_version/bispectrum.cu:221-291,
// 602-719) with every z-only factor hoisted into the node table
// (tp_tables.cu: k_node_coefs) and every triangle-shape factor (r1, r2,
// F2_tree) hoisted into the per-point record. Templated on the arithmetic
// type: double is the plain FP64 path; float uses the SFU approximations
// ex2/lg2/rcp.approx and is summed with Kahan compensation by its callers.
#pragma once
#include <type_traits>

#include "tp_internal.cuh"

namespace tp {

template <typename R>
struct Mth;
template <>
struct Mth<float> {
  static __device__ __forceinline__ float ex2(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float lg2(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
};
template <>
struct Mth<double> {
  static __device__ __forceinline__ double ex2(double x) { return exp2(x); }
  static __device__ __forceinline__ double lg2(double x) { return log2(x); }
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
};

// Cosmology constants of the integrands in arithmetic type R.
template <typename R>
struct CosmoK {
  R omh2, sa, one_m_sa, sh043, theta2, l2theta2, c184, ehc, ns, alpha_max;
  R l2h;             // log2(h)
  R h;
  int pk_given;
  R ln_kmin, inv_dk;  // tabulated P(k)
  // log2(ell) range for which every fixed line-of-sight node's P(k) table
  // coordinate lies inside the table (set with the node table; the packed
  // node-pair path clamps log2(ell) into it once per point instead of
  // clamping the coordinate at every node)
  R lgp_lo, lgp_hi;
  const double* pk;   // 256 values (FP64, read through the cache)
  const float* plt;   // log2 P_lin cubic segments (PLT_N float4) for the FP32 path, or null
};

template <typename R>
__host__ __device__ inline CosmoK<R> make_cosmok(const EHConst& e, const CosmoDev& c, const double* pk_dev) {
  CosmoK<R> k;
  k.omh2 = (R)e.omh2;
  k.sa = (R)e.sa;
  k.one_m_sa = (R)e.one_m_sa;
  k.sh043 = (R)(0.43 * e.sh);
  k.theta2 = (R)e.theta2;
  k.l2theta2 = (R)log2(e.theta2);
  k.c184 = (R)e.c184;
  k.ehc = (R)e.ehc;
  k.ns = (R)e.ns;
  k.alpha_max = (R)(1. - (2. / 3.) * c.ns);
  k.l2h = (R)log2(c.h);
  k.h = (R)c.h;
  k.pk_given = c.pk_given;
  k.ln_kmin = (R)(c.pk_given ? log(c.kmin) : 0.0);
  k.inv_dk = (R)(c.pk_given ? 1.0 / c.dk : 0.0);
  k.pk = pk_dev;
  k.plt = nullptr;
  k.lgp_lo = (R)-1e30;
  k.lgp_hi = (R)1e30;
  return k;
}

// Linear P(k) at kk = k*h [1/Mpc] with l2kk = log2(kk) (bispectrum.cu:602-693).
template <typename R>
__device__ __forceinline__ R plin(const CosmoK<R>& K, R kk, R l2kk) {
  typedef Mth<R> M;
  if (K.pk_given) {
    // table in k [h/Mpc], linear interpolation in ln k
    R lnk = (l2kk - K.l2h) * (R)LN2;
    R didx = (lnk - K.ln_kmin) * K.inv_dk;
    if (didx <= (R)0) return (R)K.pk[0];
    if (didx >= (R)(NK - 1)) return (R)K.pk[NK - 1];
    int idx = (int)didx;
    R f = didx - (R)idx;
    return (R)K.pk[idx] * ((R)1 - f) + (R)K.pk[idx + 1] * f;
  }
  if constexpr (sizeof(R) == 4) {
    if (K.plt) {
      const float inv = (float)((PLT_N - 1) / (PLT_HI - PLT_LO));
      float t = (l2kk - (float)PLT_LO) * inv;
      t = fminf(fmaxf(t, 0.f), (float)(PLT_N - 1) - 1e-3f);
      int i = (int)t;
      float f = t - (float)i;
      const float4 q = reinterpret_cast<const float4*>(K.plt)[i];
      return M::ex2(q.x + f * (q.y + f * (q.z + f * q.w)));
    }
  }
  R x = kk * K.sh043;
  R x2 = x * x;
  R geff = K.omh2 * (K.sa + K.one_m_sa * M::rcp((R)1 + x2 * x2));
  R l2q = l2kk + K.l2theta2 - M::lg2(geff);
  R qe = M::ex2(l2q);
  R q111 = M::ex2((R)1.11 * l2q);
  R L = (R)LN2 * M::lg2((R)2.718281828 + K.c184 * qe);
  R C = (R)14.4 + (R)325.0 * M::rcp((R)1 + (R)60.5 * q111);
  R r = L * M::rcp(L + C * qe * qe);
  return K.ehc * M::ex2(K.ns * l2kk) * r * r;
}

// Triangle record shared by all nodes of one b_kappa evaluation.
template <typename R>
struct Tri {
  R l[3];      // ell_i
  R lg[3];     // log2 ell_i
  R log2r1;    // log2(ell_min/ell_max)
  R r2sq;      // r2^2, r2 = (ell_mid + ell_min - ell_max)/ell_max
  R pr2;       // 10^(0.007 r2)
  R f2t[3];    // F2_tree(1,2,3), F2_tree(2,3,1), F2_tree(3,1,2)
};

__host__ __device__ inline double f2_tree(double k1, double k2, double k3) {
  double c12 = 0.5 * (k3 * k3 - k1 * k1 - k2 * k2) / (k1 * k2);
  return (5. / 7.) + 0.5 * c12 * (k1 / k2 + k2 / k1) + (2. / 7.) * c12 * c12;
}

template <typename R>
__device__ inline void make_tri(double l1, double l2, double l3, Tri<R>& T) {
  T.l[0] = (R)l1;
  T.l[1] = (R)l2;
  T.l[2] = (R)l3;
  T.lg[0] = (R)log2(l1);
  T.lg[1] = (R)log2(l2);
  T.lg[2] = (R)log2(l3);
  double a = l1, b = l2, c = l3, t;
  if (a < b) { t = a; a = b; b = t; }
  if (a < c) { t = a; a = c; c = t; }
  if (b < c) { t = b; b = c; c = t; }
  // a >= b >= c (bispectrum.cu:235-247)
  double r1 = c / a, r2 = (b + c - a) / a;
  T.log2r1 = (R)log2(r1);
  T.r2sq = (R)(r2 * r2);
  T.pr2 = (R)exp2(LOG2_10 * 0.007 * r2);
  T.f2t[0] = (R)f2_tree(l1, l2, l3);
  T.f2t[1] = (R)f2_tree(l2, l3, l1);
  T.f2t[2] = (R)f2_tree(l3, l1, l2);
}

// FP32 triangle setup from (l1, l2, phi) of the <Map^3> parametrisation
// (l3^2 = l1^2 + l2^2 + 2 l1 l2 cos phi), written without cancellation:
// l3^2 = (l1-l2)^2 + 4 l1 l2 cos^2(phi/2), and the three F2_tree cosines from
// the closed triangle l1 + l2 + l3 = 0: cos12 = cos phi,
// cos23 = -(l1 cos phi + l2)/l3, cos31 = -(l1 + l2 cos phi)/l3.
__device__ __forceinline__ float f2t_cos(float c, float a, float b) {
  return (5.f / 7.f) + 0.5f * c * (a / b + b / a) + (2.f / 7.f) * c * c;
}
__device__ __forceinline__ void make_tri_phi_f(float l1, float l2, float cphi, float l3, Tri<float>& T) {
  typedef Mth<float> M;
  T.l[0] = l1;
  T.l[1] = l2;
  T.l[2] = l3;
  T.lg[0] = M::lg2(l1);
  T.lg[1] = M::lg2(l2);
  T.lg[2] = M::lg2(l3);
  float a = l1, b = l2, c = l3, la = T.lg[0], lb = T.lg[1], lc = T.lg[2], t;
  if (a < b) { t = a; a = b; b = t; t = la; la = lb; lb = t; }
  if (a < c) { t = a; a = c; c = t; t = la; la = lc; lc = t; }
  if (b < c) { t = b; b = c; c = t; t = lb; lb = lc; lc = t; }
  float ia = M::rcp(a);
  float r2 = (b + c - a) * ia;
  T.log2r1 = lc - la;
  T.r2sq = r2 * r2;
  T.pr2 = M::ex2((float)(LOG2_10 * 0.007) * r2);
  float il3 = M::rcp(l3);
  float c23 = -(l1 * cphi + l2) * il3;
  float c31 = -(l1 + l2 * cphi) * il3;
  T.f2t[0] = f2t_cos(cphi, l1, l2);
  T.f2t[1] = f2t_cos(c23, l2, l3);
  T.f2t[2] = f2t_cos(c31, l3, l1);
}

// B at one redshift from its coefficient vector nc[c * stride] (c = NC_*),
// for a triangle whose ell_i = T.l[i] * sc (log2: T.lg[i] + l2sc):
// q_i = ell_i * s, k_i h = ell_i * hf.
template <typename R>
__device__ __forceinline__ R bispec_eval(const R* __restrict__ nc, int stride, R s, R l2s, R hf, R l2hf,
                                         const Tri<R>& T, const CosmoK<R>& K) {
  typedef Mth<R> M;
#define NCV(c) nc[(c) * stride]
  R q[3], lq[3], P[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    q[i] = T.l[i] * s;
    lq[i] = T.lg[i] + l2s;
  }
  if (NCV(NC_TREE) != (R)0) {
    // tree level for z > 10 (bispectrum.cu:229-230,695-698)
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = plin<R>(K, T.l[i] * hf, T.lg[i] + l2hf);
    return NCV(NC_D1P4) * (R)2 * (T.f2t[0] * P[0] * P[1] + T.f2t[1] * P[1] * P[2] + T.f2t[2] * P[2] * P[0]);
  }
  // 1-halo term (B4, B7)
  const R an = M::ex2(NCV(NC_ANA) - NCV(NC_ANR) * M::ex2(NCV(NC_ANC) * T.log2r1));
  R al = M::ex2(NCV(NC_ALA) + NCV(NC_ALD) * T.r2sq);
  al = al > K.alpha_max ? K.alpha_max : al;
  const R be = NCV(NC_BETAB) * T.pr2;
  const R bn = NCV(NC_BN), cn = NCV(NC_CN);
  R bs1h = (R)1;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R cq = cn * q[i];
    bs1h *= cq * M::rcp((an * M::ex2(al * lq[i]) + bn * M::ex2(be * lq[i])) * (cq + (R)1));
  }
  // 3-halo term (B5, B6, B9)
  const R fn = NCV(NC_FN), gn = NCV(NC_GN), hn = NCV(NC_HN);
  const R mn = NCV(NC_MN), nn = NCV(NC_NN);
  const R mun = NCV(NC_MUN), nun = NCV(NC_NUN);
  const R pn = NCV(NC_PN), en = NCV(NC_EN);
  const R d1sq = NCV(NC_D1SQ);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    R qi = q[i];
    R a = ((R)1 + fn * qi * qi) * M::rcp((R)1 + gn * qi + hn * qi * qi) * d1sq *
          plin<R>(K, T.l[i] * hf, T.lg[i] + l2hf);
    R x = pn * qi;
    R x3 = x * x * x;
    R mq = mn * M::ex2(mun * lq[i]) + nn * M::ex2(nun * lq[i]);
    P[i] = a + x3 * M::rcp(mq * (x3 + (R)1));
  }
  const R dn = NCV(NC_DN);
  R bs3h = (R)2 * ((T.f2t[0] + dn * q[2]) * P[0] * P[1] + (T.f2t[1] + dn * q[0]) * P[1] * P[2] +
                   (T.f2t[2] + dn * q[1]) * P[2] * P[0]);
  bs3h *= M::rcp(((R)1 + en * q[0]) * ((R)1 + en * q[1]) * ((R)1 + en * q[2]));
#undef NCV
  return bs1h + bs3h;
}

// B(ell_i / f_K(z_j), z_j) at line-of-sight node j of a node table stored
// node-major (coef c of node j at nc[j*NCP + c]); the FP32 row is fetched with
// 16-byte vector loads.
template <typename R>
__device__ __forceinline__ R bispec_node(const R* __restrict__ nc, int j, const Tri<R>& T, const CosmoK<R>& K) {
  const R* row = nc + j * NCP;
  if constexpr (sizeof(R) == 4) {
    float c[NCP];
    const float4* v = reinterpret_cast<const float4*>(row);
#pragma unroll
    for (int q = 0; q < NCP / 4; ++q) {
      float4 t = v[q];
      c[4 * q] = t.x;
      c[4 * q + 1] = t.y;
      c[4 * q + 2] = t.z;
      c[4 * q + 3] = t.w;
    }
    return c[NC_W] * bispec_eval<float>(c, 1, c[NC_S], c[NC_L2S], c[NC_HF], c[NC_L2HF], T, K);
  } else {
    return row[NC_W] * bispec_eval<R>(row, 1, row[NC_S], row[NC_L2S], row[NC_HF], row[NC_L2HF], T, K);
  }
}

// ---------------------------------------------------------------------------
// FP32 point path of <Map^3> and b_kappa: NF_* node rows (tp_internal.cuh).
// Per triangle it keeps ell_i^2 besides the Tri fields; the record is 15 words.
struct TriF {
  float l[3], lg[3], l2[3];
  float log2r1, r2sq, pr2;
  float f2t[3];
};

__device__ __forceinline__ void trif_from_tri(const Tri<float>& T, TriF& F) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    F.l[i] = T.l[i];
    F.lg[i] = T.lg[i];
    F.l2[i] = T.l[i] * T.l[i];
    F.f2t[i] = T.f2t[i];
  }
  F.log2r1 = T.log2r1;
  F.r2sq = T.r2sq;
  F.pr2 = T.pr2;
}

// P_lin(ell h / f_K) from the node's row: the cubic log2 P table when present
// (table coordinate lg * (N-1)/(HI-LO) + NF_TOFF; the integer part by a
// round-down add of 1.5 * 2^23, no float/int conversions), else plin().
__device__ __forceinline__ float plin_fast(const CosmoK<float>& K, const float* __restrict__ c, float l, float lg) {
  typedef Mth<float> M;
  if (K.plt) {
    constexpr float INV = (float)((PLT_N - 1) / (PLT_HI - PLT_LO));
    float t = fmaf(lg, INV, c[NF_TOFF]);
    t = fminf(fmaxf(t, 0.f), (float)(PLT_N - 1) - 1e-3f);
    const float tm = __fadd_rd(t, 12582912.f);  // 1.5 * 2^23 + floor(t)
    const int i = __float_as_int(tm) - 0x4B400000;
    const float f = t - (tm - 12582912.f);
    const float4 q = reinterpret_cast<const float4*>(K.plt)[i];
    return M::ex2(fmaf(f, fmaf(f, fmaf(f, q.w, q.z), q.y), q.x));
  }
  return plin<float>(K, l * c[NF_HF], lg + c[NF_L2HF]);
}

// plin<float> kept out of line: the tabulated-P(k) and Eisenstein & Hu
// branches are not taken when the cubic table exists, and inlined they hold
// a dozen cosmology constants in registers across the node loops
static __device__ __noinline__ float plin_outline(const CosmoK<float>* K, float kk, float l2kk) {
  return plin<float>(*K, kk, l2kk);
}

// ---- packed FP32 pairs (fma/mul/add .f32x2: one issue slot for two lanes) --
__device__ __forceinline__ float2 p2fma(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 p2mul(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 p2add(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 p2sub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 p2add_rd(float2 a, float2 b) {  // rounded toward -inf
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rm.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 p2dup(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 p2ex2(float2 a) { return make_float2(Mth<float>::ex2(a.x), Mth<float>::ex2(a.y)); }
__device__ __forceinline__ float2 p2rcp(float2 a) { return make_float2(Mth<float>::rcp(a.x), Mth<float>::rcp(a.y)); }

// The triangle of TriF with every field duplicated into both lanes of a pair.
struct TriF2 {
  float2 l[3], lg[3], l2[3];
  float2 log2r1, r2sq, pr2;
  float2 f2t[3];
  float2 lgp[3];  // log2 ell_i clamped into [lgp_lo, lgp_hi] (P(k) table lookups only)
};
__device__ __forceinline__ void trif2_from(const TriF& T, TriF2& D, float lgp_lo, float lgp_hi) {
#pragma unroll
  for (int i = 0; i < 3; ++i) D.lgp[i] = p2dup(fminf(fmaxf(T.lg[i], lgp_lo), lgp_hi));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    D.l[i] = p2dup(T.l[i]);
    D.lg[i] = p2dup(T.lg[i]);
    D.l2[i] = p2dup(T.l2[i]);
    D.f2t[i] = p2dup(T.f2t[i]);
  }
  D.log2r1 = p2dup(T.log2r1);
  D.r2sq = p2dup(T.r2sq);
  D.pr2 = p2dup(T.pr2);
}

// NF_* tables are stored as node pairs: coefficient k of node j at float
// index ((j / 2) * NCP + k) * 2 + (j % 2), so that a pair's coefficient is
// one float2 (the two lanes of the packed evaluation).
__device__ __forceinline__ int nf_index(int j, int k) { return ((j >> 1) * NCP + k) * 2 + (j & 1); }

// B at one node (the bispec_eval formula, B4-B9 of Takahashi et al. 2020,
// with the folded NF_* coefficients) for the two nodes of pair c (c[k] =
// coefficient k of both nodes), W not applied. Lanes are independent: the .x
// lane is node 2p, the .y lane node 2p+1.
// The triangle is a TriF2 (pairs held in registers) or a TriF (each value
// duplicated where it is used): v2() gives the pair either way.
__device__ __forceinline__ float2 v2(float x) { return p2dup(x); }
__device__ __forceinline__ float2 v2(float2 x) { return x; }

// MERGE: one reciprocal for the three 1-halo denominators and one per 3-halo
// side for both of its fractions (10 fewer MUFU per pair). A merged product
// that overflows makes the node NaN (the product times 0 is added), and one
// that falls below the normal range gives rcp = inf, so every such case shows
// as a non-finite node; the caller then re-evaluates with MERGE = false.
template <class TT, bool MERGE = false>
__device__ __forceinline__ float2 bispec_pair(const float2* __restrict__ c, const TT& T, const CosmoK<float>& K) {
  typedef Mth<float> M;
  const float2 one = p2dup(1.f);
  float2 lq[3], P[3];
  const float2 l2s = c[NF_L2S];
#pragma unroll
  for (int i = 0; i < 3; ++i) lq[i] = p2add(v2(T.lg[i]), l2s);
  const float2 tree = c[NF_TREE];
  if (tree.x != 0.f || tree.y != 0.f) {
    // tree level beyond z = 10 (both lanes evaluated the same way)
    const float2 d1p4 = c[NF_D1P4];
    float2 r;
    const float* cf = reinterpret_cast<const float*>(c);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float Ps[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float li = h ? v2(T.l[i]).y : v2(T.l[i]).x, lgi = h ? v2(T.lg[i]).y : v2(T.lg[i]).x;
        float cl[NCP];
#pragma unroll
        for (int k = 0; k < NCP; ++k) cl[k] = cf[2 * k + h];
        Ps[i] = plin_fast(K, cl, li, lgi);
      }
      const float f0 = v2(T.f2t[0]).x, f1 = v2(T.f2t[1]).x, f2 = v2(T.f2t[2]).x;
      const float v = (h ? d1p4.y : d1p4.x) * 2.f * (f0 * Ps[0] * Ps[1] + f1 * Ps[1] * Ps[2] + f2 * Ps[2] * Ps[0]);
      if (h) r.y = v; else r.x = v;
    }
    return r;
  }
  // 1-halo term: 1 / ((a_n q^al + b_n q^be) (1 + 1/(c_n q))) per side
  const float2 l2an = p2sub(c[NF_ANA], p2ex2(p2fma(c[NF_ANC], v2(T.log2r1), c[NF_L2ANR])));
  float2 al = p2ex2(p2fma(c[NF_ALD], v2(T.r2sq), c[NF_ALA]));
  al.x = fminf(al.x, K.alpha_max);
  al.y = fminf(al.y, K.alpha_max);
  const float2 be = p2mul(c[NF_BETAB], v2(T.pr2));
  const float2 cns = c[NF_CNS], l2bn = c[NF_L2BN];
  const float2 zero = p2dup(0.f);
  float2 bs1h = one;
  if constexpr (MERGE) {
    float2 num1 = one, den1 = one;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 cq = p2mul(cns, v2(T.l[i]));
      const float2 den = p2add(p2ex2(p2fma(al, lq[i], l2an)), p2ex2(p2fma(be, lq[i], l2bn)));
      num1 = p2mul(num1, cq);
      den1 = p2mul(den1, p2mul(den, p2add(cq, one)));
    }
    bs1h = p2fma(den1, zero, p2mul(num1, p2rcp(den1)));
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float2 cq = p2mul(cns, v2(T.l[i]));
      const float2 den = p2add(p2ex2(p2fma(al, lq[i], l2an)), p2ex2(p2fma(be, lq[i], l2bn)));
      bs1h = p2mul(bs1h, p2mul(cq, p2rcp(p2mul(den, p2add(cq, one)))));
    }
  }
  // 3-halo term
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float2 num = p2fma(c[NF_D1SQFNS2], v2(T.l2[i]), c[NF_D1SQ]);
    const float2 den = p2fma(c[NF_HNS2], v2(T.l2[i]), p2fma(c[NF_GNS], v2(T.l[i]), one));
    // linear P(k) of the two nodes (table lookups per lane)
    float2 pl;
    {
      constexpr float INV = (float)((PLT_N - 1) / (PLT_HI - PLT_LO));
      constexpr bool pre = std::is_same<TT, TriF2>::value;  // log2 ell already clamped per point
      float2 t2;
      if constexpr (pre)
        t2 = p2fma(T.lgp[i], p2dup(INV), c[NF_TOFF]);
      else
        t2 = p2fma(v2(T.lg[i]), p2dup(INV), c[NF_TOFF]);
      if (K.plt) {
        float2 tc = t2;
        if constexpr (!pre) {
          tc.x = fminf(fmaxf(tc.x, 0.f), (float)(PLT_N - 1) - 1e-3f);
          tc.y = fminf(fmaxf(tc.y, 0.f), (float)(PLT_N - 1) - 1e-3f);
        }
        // floor and fraction of both lanes with packed adds: tm = 1.5 * 2^23 + floor(t)
        const float2 big = p2dup(12582912.f);
        const float2 tm = p2add_rd(tc, big);
        const float2 f2 = p2sub(tc, p2sub(tm, big));
        const float tf[2] = {f2.x, f2.y};
        const int ixs[2] = {__float_as_int(tm.x) - 0x4B400000, __float_as_int(tm.y) - 0x4B400000};
        float r[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const float f = tf[h];
          const float4 q = reinterpret_cast<const float4*>(K.plt)[ixs[h]];
          r[h] = M::ex2(fmaf(f, fmaf(f, fmaf(f, q.w, q.z), q.y), q.x));
        }
        pl = make_float2(r[0], r[1]);
      } else {
        const float2 hf = c[NF_HF], l2hf = c[NF_L2HF];
        pl.x = plin_outline(&K, v2(T.l[i]).x * hf.x, v2(T.lg[i]).x + l2hf.x);
        pl.y = plin_outline(&K, v2(T.l[i]).y * hf.y, v2(T.lg[i]).y + l2hf.y);
      }
    }
    const float2 x = p2mul(c[NF_PNS], v2(T.l[i]));
    const float2 x3 = p2mul(p2mul(x, x), x);
    const float2 mq = p2add(p2ex2(p2fma(c[NF_MUN], lq[i], c[NF_L2MN])), p2ex2(p2fma(c[NF_NUN], lq[i], c[NF_L2NN])));
    if constexpr (MERGE) {
      // num pl / den + x^3 / M = (x^3 den + num pl M) / (den M),  M = mq (1 + x^3)
      const float2 M = p2mul(mq, p2add(x3, one));
      const float2 dm = p2mul(den, M);
      const float2 t = p2fma(x3, den, p2mul(p2mul(num, pl), M));
      P[i] = p2fma(dm, zero, p2mul(t, p2rcp(dm)));
    } else {
      const float2 a = p2mul(p2mul(num, p2rcp(den)), pl);
      P[i] = p2fma(x3, p2rcp(p2mul(mq, p2add(x3, one))), a);
    }
  }
  const float2 dn = c[NF_DNS], en = c[NF_ENS];
  float2 bs3h = p2mul(p2mul(p2fma(dn, v2(T.l[2]), v2(T.f2t[0])), P[0]), P[1]);
  bs3h = p2fma(p2mul(p2fma(dn, v2(T.l[0]), v2(T.f2t[1])), P[1]), P[2], bs3h);
  bs3h = p2fma(p2mul(p2fma(dn, v2(T.l[1]), v2(T.f2t[2])), P[2]), P[0], bs3h);
  const float2 e3 = p2mul(p2mul(p2fma(en, v2(T.l[0]), one), p2fma(en, v2(T.l[1]), one)), p2fma(en, v2(T.l[2]), one));
  return p2fma(p2mul(p2dup(2.f), bs3h), p2rcp(e3), bs1h);
}

// W B at the two nodes of pair p of a pair-interleaved NF_* table
template <class TT, bool MERGE = false>
__device__ __forceinline__ float2 bispec_pair_node(const float* __restrict__ nf, int p, const TT& T,
                                                   const CosmoK<float>& K) {
  const float2* c = reinterpret_cast<const float2*>(nf) + (size_t)p * NCP;
  return p2mul(c[NF_W], bispec_pair<TT, MERGE>(c, T, K));
}

// B from one NF_* row c[0..NF_COUNT) (the scalar form of bispec_pair), W not applied
__device__ __forceinline__ float bispec_fast_row(const float* c, const TriF& T, const CosmoK<float>& K) {
  typedef Mth<float> M;
  float lq[3], P[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) lq[i] = T.lg[i] + c[NF_L2S];
  float B;
  if (c[NF_TREE] != 0.f) {
#pragma unroll
    for (int i = 0; i < 3; ++i) P[i] = plin_fast(K, c, T.l[i], T.lg[i]);
    B = c[NF_D1P4] * 2.f * (T.f2t[0] * P[0] * P[1] + T.f2t[1] * P[1] * P[2] + T.f2t[2] * P[2] * P[0]);
  } else {
    const float l2an = c[NF_ANA] - M::ex2(fmaf(c[NF_ANC], T.log2r1, c[NF_L2ANR]));
    const float al = fminf(M::ex2(fmaf(c[NF_ALD], T.r2sq, c[NF_ALA])), K.alpha_max);
    const float be = c[NF_BETAB] * T.pr2;
    float bs1h = 1.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float cq = c[NF_CNS] * T.l[i];
      const float den = M::ex2(fmaf(al, lq[i], l2an)) + M::ex2(fmaf(be, lq[i], c[NF_L2BN]));
      bs1h *= cq * M::rcp(den * (cq + 1.f));
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float num = fmaf(c[NF_D1SQFNS2], T.l2[i], c[NF_D1SQ]);
      const float den = fmaf(c[NF_HNS2], T.l2[i], fmaf(c[NF_GNS], T.l[i], 1.f));
      const float a = num * M::rcp(den) * plin_fast(K, c, T.l[i], T.lg[i]);
      const float x = c[NF_PNS] * T.l[i];
      const float x3 = x * x * x;
      const float mq = M::ex2(fmaf(c[NF_MUN], lq[i], c[NF_L2MN])) + M::ex2(fmaf(c[NF_NUN], lq[i], c[NF_L2NN]));
      P[i] = fmaf(x3, M::rcp(mq * (x3 + 1.f)), a);
    }
    const float dn = c[NF_DNS], en = c[NF_ENS];
    float bs3h = fmaf(dn, T.l[2], T.f2t[0]) * P[0] * P[1];
    bs3h = fmaf(fmaf(dn, T.l[0], T.f2t[1]) * P[1], P[2], bs3h);
    bs3h = fmaf(fmaf(dn, T.l[1], T.f2t[2]) * P[2], P[0], bs3h);
    const float e3 = fmaf(en, T.l[0], 1.f) * fmaf(en, T.l[1], 1.f) * fmaf(en, T.l[2], 1.f);
    B = fmaf(2.f * bs3h, M::rcp(e3), bs1h);
  }
  return B;
}

// W B at node j of a pair-interleaved NF_* table, one lane per node
__device__ __forceinline__ float bispec_node_fast(const float* __restrict__ nf, int j, const TriF& T,
                                                  const CosmoK<float>& K) {
  float c[NCP];
#pragma unroll
  for (int k = 0; k < NCP; ++k) c[k] = nf[nf_index(j, k)];
  return c[NF_W] * bispec_fast_row(c, T, K);
}

// NF_* row of one arbitrary redshift from its NC_* coefficients zc (zcoefs):
// the folding of k_node_coefs, for integrands whose redshift varies per point.
__device__ __forceinline__ void nf_from_nc(const float* zc, float* nf) {
  typedef Mth<float> M;
  const float s = zc[NC_S];
  nf[NF_W] = zc[NC_W];
  nf[NF_L2S] = zc[NC_L2S];
  nf[NF_L2HF] = zc[NC_L2HF];
  nf[NF_HF] = zc[NC_HF];
  nf[NF_TOFF] = (zc[NC_L2HF] - (float)PLT_LO) * (float)((PLT_N - 1) / (PLT_HI - PLT_LO));
  nf[NF_ANA] = zc[NC_ANA];
  nf[NF_L2ANR] = M::lg2(zc[NC_ANR]);
  nf[NF_ANC] = zc[NC_ANC];
  nf[NF_L2BN] = M::lg2(zc[NC_BN]);
  nf[NF_CNS] = zc[NC_CN] * s;
  nf[NF_ALA] = zc[NC_ALA];
  nf[NF_ALD] = zc[NC_ALD];
  nf[NF_BETAB] = zc[NC_BETAB];
  nf[NF_D1SQ] = zc[NC_D1SQ];
  nf[NF_D1SQFNS2] = zc[NC_D1SQ] * zc[NC_FN] * s * s;
  nf[NF_GNS] = zc[NC_GN] * s;
  nf[NF_HNS2] = zc[NC_HN] * s * s;
  nf[NF_L2MN] = M::lg2(zc[NC_MN]);
  nf[NF_L2NN] = M::lg2(zc[NC_NN]);
  nf[NF_MUN] = zc[NC_MUN];
  nf[NF_NUN] = zc[NC_NUN];
  nf[NF_PNS] = zc[NC_PN] * s;
  nf[NF_ENS] = zc[NC_EN] * s;
  nf[NF_DNS] = zc[NC_DN] * s;
  nf[NF_TREE] = zc[NC_TREE];
  nf[NF_D1P4] = zc[NC_D1P4];
#pragma unroll
  for (int k = NF_COUNT; k < NCP; ++k) nf[k] = 0.f;
}

// the triangle scaled by sc (log2 l2sc): ell_i -> ell_i sc; shape factors unchanged
__device__ __forceinline__ TriF trif_scaled(const TriF& T, float sc, float l2sc) {
  TriF S = T;
  const float sc2 = sc * sc;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.l[i] = T.l[i] * sc;
    S.l2[i] = T.l2[i] * sc2;
    S.lg[i] = T.lg[i] + l2sc;
  }
  return S;
}

// Mid-bin two-point interpolation of a z table at fractional bin position fb
// (cuda_version/bispectrum.cu:335-437) with the lower neighbour clamped at bin 0.
__host__ __device__ inline void interp_mid_w(double fb, int& i0, int& i1, double& w0, double& w1) {
  int idx = (int)fb;
  double didx = fb - idx;
  if (idx > NZ - 1) {
    idx = NZ - 1;
    didx = 1.0;
  }
  int ii = idx;
  double w = 1 - fabs(didx - 0.5), iw = 1 - w;
  if (didx > 0.5) {
    if (idx == NZ - 1)
      iw = 0.0;
    else
      ii = idx + 1;
  } else if (didx < 0.5) {
    ii = idx - 1 < 0 ? 0 : idx - 1;
  }
  i0 = idx;
  i1 = ii;
  w0 = w;
  w1 = iw;
}

// BiHalofit coefficients of one arbitrary redshift z (the z-only part of
// integrand_bkappa + bispec, bispectrum.cu:221-333), into zc[NC_*] with
// NC_W = (g(1+z))^3 / f_K / E(z) (no quadrature weight). Returns false when
// integrand_bkappa is zero at this z (z < 1e-7).
template <typename R>
__device__ inline bool zcoefs(const TablesDev& t, const CosmoDev& c, double z, R* zc) {
  if (z < 1.0e-7) return false;
  int i0, i1;
  double w0, w1;
  interp_mid_w(z / c.zmax * NZ, i0, i1, w0, w1);
  double g = t.g[i0] * w0 + t.g[i1] * w1, fK = t.f_K[i0] * w0 + t.f_K[i1] * w1;
  double D1 = t.D1[i0] * w0 + t.D1[i1] * w1, rs = t.r_sigma[i0] * w0 + t.r_sigma[i1] * w1;
  double ned = t.n_eff[i0] * w0 + t.n_eff[i1] * w1;
  typedef Mth<R> M;
  const R L10 = (R)LOG2_10;
  R zp = (R)(1.0 + z);
  R l2zp = M::lg2(zp);
  R E = sqrt((R)c.om * zp * zp * zp + (R)c.ow * M::ex2((R)(3 * (1.0 + c.w)) * l2zp));
  R gz = (R)g * zp;
  R fKr = (R)fK;
  zc[NC_W] = gz * gz * gz / fKr / E;
  R sr = (R)(rs / fK);
  zc[NC_S] = sr;
  zc[NC_L2S] = M::lg2(sr);
  R hf = (R)(c.h / fK);
  zc[NC_HF] = hf;
  zc[NC_L2HF] = M::lg2(hf);
  R ls = M::lg2((R)(D1 * c.sigma8)) * (R)0.30102999566398119521;
  R ne = (R)ned;
  R aexp = M::ex2((R)(-3. * c.w) * (-l2zp));  // a^(-3w), a = 1/(1+z)
  R omz = (R)c.om / ((R)c.om + (R)c.ow * aexp);
  zc[NC_ANA] = L10 * ((R)-2.167 + ls * ((R)-2.944 + ls * ((R)-1.106 + ls * (R)-2.865)));
  zc[NC_ANR] = (R)(0.310 * LOG2_10);
  zc[NC_ANC] = M::ex2(L10 * ((R)0.182 + (R)0.57 * ne));
  zc[NC_BN] = M::ex2(L10 * ((R)-3.428 + ls * ((R)-2.681 + ls * ((R)1.624 + ls * (R)-0.095))));
  zc[NC_CN] = M::ex2(L10 * ((R)0.159 - (R)1.107 * ne));
  zc[NC_ALA] = L10 * ((R)-4.348 + ne * ((R)-3.006 + ne * (R)-0.5745));
  zc[NC_ALD] = L10 * M::ex2(L10 * ((R)-0.9 + (R)0.2 * ne));
  zc[NC_BETAB] = M::ex2(L10 * ((R)-1.731 + ne * ((R)-2.845 + ne * ((R)-1.4995 + ne * (R)-0.2811))));
  zc[NC_FN] = M::ex2(L10 * ((R)-10.533 + ne * ((R)-16.838 + ne * ((R)-9.3048 + ne * (R)-1.8263))));
  zc[NC_GN] = M::ex2(L10 * ((R)2.787 + ne * ((R)2.405 + ne * (R)0.4577)));
  zc[NC_HN] = M::ex2(L10 * ((R)-1.118 - (R)0.394 * ne));
  zc[NC_MN] = M::ex2(L10 * ((R)-2.605 + ls * ((R)-2.434 + ls * (R)5.71)));
  zc[NC_NN] = M::ex2(L10 * ((R)-4.468 + ls * ((R)-3.08 + ls * (R)1.035)));
  zc[NC_MUN] = M::ex2(L10 * ((R)15.312 + ne * ((R)22.977 + ne * ((R)10.9579 + ne * (R)1.6586))));
  zc[NC_NUN] = M::ex2(L10 * ((R)1.347 + ne * ((R)1.246 + ne * (R)0.4525)));
  zc[NC_PN] = M::ex2(L10 * ((R)0.071 - (R)0.433 * ne));
  zc[NC_EN] = M::ex2(L10 * ((R)-0.632 + (R)0.646 * ne));
  zc[NC_DN] = M::ex2(L10 * ((R)-0.483 + (R)0.892 * ls - (R)0.086 * omz));
  R d1 = (R)D1;
  zc[NC_D1SQ] = d1 * d1;
  zc[NC_TREE] = z > 10. ? (R)1 : (R)0;
  zc[NC_D1P4] = d1 * d1 * d1 * d1;
  return true;
}

__device__ __forceinline__ double uhat(double eta) {
  double t = 0.5 * eta * eta;
  return t * exp(-t);
}

// Kahan accumulator
template <typename R>
struct KSum {
  R s = 0, c = 0;
  __device__ __forceinline__ void add(R v) {
    R y = v - c;
    R t = s + y;
    c = (t - s) - y;
    s = t;
  }
};
template <>
struct KSum<double> {
  double s = 0;
  __device__ __forceinline__ void add(double v) { s += v; }
};

}  // namespace tp
