// Device-side h-adaptive cubature for batches of independent integrals.
//
// Semantics follow the reference's vendored Gladwell-parallel hcubature_v
// (cuda_version/hcubature.cpp:456-617 rule, 620-780 1-D rule, 904-1067
// driver; converged.h): every sweep evaluates all regions split in the
// previous sweep; a sweep splits the largest-error regions, in decreasing
// order of their maximum component error, until the remaining error meets the
// tolerance; a region is halved along the dimension of largest fourth
// difference; the lower half keeps the parent volume * 0.5 and the upper half
// recomputes the product of its widths.
//
// GB300 mapping: one CTA owns one integral for its whole adaptive life (a
// persistent grid pulls integrals from an atomic job counter), so no CTA ever
// waits on another; for small batches the CTAs of a thread-block cluster own
// one integral together (adaptive_body with CS > 1, below), synchronised by
// the hardware cluster barrier only. Region state lives in a per-CTA (per
// cluster) slot of HBM scratch (structure of arrays, FP64). Inside a sweep the CTA evaluates the new
// regions' cubature points in chunks; each point's integrand is split into G
// independent partial sums (for the line-of-sight integrands: G groups of
// nodes), giving (point x group) parallelism even for one-region sweeps. The
// region choice is a radix select on the bit pattern of the FP64 error keys
// (8 passes of 256-bin shared-memory histograms) followed by a block-wide
// stream compaction; no sort and no host round trip.
#pragma once
#include <cooperative_groups.h>
#include <stdint.h>

#include "tp_internal.cuh"

namespace tp {

// Genz-Malik generators sqrt(9/70), sqrt(9/10), sqrt(9/19) (correctly rounded)
// and ratio = l2^2 / l4^2 as computed in double from them.
struct GM {
  static constexpr double l2 = 0x1.6f2c9a420071ep-2;
  static constexpr double l4 = 0x1.e5b9d136c6d96p-1;
  static constexpr double l5 = 0x1.6061efecf8ae9p-1;
  static constexpr double ratio = 0x1.2492492492493p-3;
};

// 15-point Kronrod abscissae, 7-point Gauss weights and 15-point Kronrod
// weights (QUADPACK qk15 constants)
__device__ __forceinline__ double gk_xgk(int i) {
  const double v[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                       0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                       0.586087235467691130294144838258730, 0.405845151377397166906606412076961,
                       0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
  return v[i];
}
__device__ __forceinline__ double gk_wg(int i) {
  const double v[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                       0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
  return v[i];
}
__device__ __forceinline__ double gk_wgk(int i) {
  const double v[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                       0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                       0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                       0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
  return v[i];
}

template <int DIM>
struct GMRule {
  static constexpr int NP = (DIM == 1) ? 15 : 1 + 4 * DIM + 2 * DIM * (DIM - 1) + (1 << DIM);
};

struct EngineCfg {
  double abs_tol, rel_tol;
  int norm;        // TP_NORM_*; fdim == 1 always behaves as INDIVIDUAL
  int cap;         // regions per integral
  int max_sweeps;
};

// per-CTA region store
template <int DIM, int FDIM>
struct Slot {
  double* cen;    // [DIM][cap]
  double* hw;     // [DIM][cap]
  double* vol;    // [cap]
  double* val;    // [FDIM][cap]
  double* err;    // [FDIM][cap]
  double* emax;   // [cap]
  int* pend;      // [cap]
  uint8_t* split; // [cap]
  int cap;
  __host__ __device__ static constexpr size_t bytes(int cap) {
    return (size_t)cap * (sizeof(double) * (2 * DIM + 2 + 2 * FDIM) + sizeof(int) + 1) + 256;
  }
  __device__ void init(char* base, int c) {
    cap = c;
    double* d = (double*)base;
    cen = d;
    hw = cen + (size_t)DIM * cap;
    vol = hw + (size_t)DIM * cap;
    val = vol + cap;
    err = val + (size_t)FDIM * cap;
    emax = err + (size_t)FDIM * cap;
    pend = (int*)(emax + cap);
    split = (uint8_t*)(pend + cap);
  }
};

// ---------------------------------------------------------------------------
// cubature point p of a region (same ordering as the reference rules)
template <int DIM>
__device__ inline void rule_point(int p, const double* c, const double* h, double* x) {
#pragma unroll
  for (int d = 0; d < DIM; ++d) x[d] = c[d];
  if constexpr (DIM == 1) {
    // center, then +-xgk[1], +-xgk[3], +-xgk[5], then +-xgk[0], +-xgk[2], +-xgk[4], +-xgk[6]
    if (p == 0) return;
    int q = p - 1;
    int j = q >> 1;
    int idx = j < 3 ? 2 * j + 1 : 2 * (j - 3);
    double w = h[0] * gk_xgk(idx);
    x[0] = (q & 1) ? c[0] + w : c[0] - w;
  } else {
    if (p == 0) return;
    if (p < 1 + 4 * DIM) {
      int k = (p - 1) >> 2, s = (p - 1) & 3;
      double r = (s < 2 ? GM::l2 : GM::l4) * h[k];
      x[k] = (s & 1) ? c[k] + r : c[k] - r;
      return;
    }
    int q = p - (1 + 4 * DIM);
    if (q < 2 * DIM * (DIM - 1)) {
      int pr = q >> 2, s = q & 3;
      int i = 0, j = 1, cnt = 0;
      for (int a = 0; a < DIM - 1; ++a)
        for (int b = a + 1; b < DIM; ++b) {
          if (cnt == pr) {
            i = a;
            j = b;
          }
          ++cnt;
        }
      double ri = GM::l4 * h[i], rj = GM::l4 * h[j];
      // (-,-), (+,-), (+,+), (-,+)
      x[i] = (s == 1 || s == 2) ? c[i] + ri : c[i] - ri;
      x[j] = (s >= 2) ? c[j] + rj : c[j] - rj;
      return;
    }
    int m = q - 2 * DIM * (DIM - 1);
    int gray = m ^ (m >> 1);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double r = GM::l5 * h[d];
      x[d] = ((gray >> d) & 1) ? c[d] - r : c[d] + r;
    }
  }
}

// Apply the embedded rule to one region's NP point values (f[p*FDIM+k]).
template <int DIM, int FDIM>
__device__ inline void rule_combine(const double* f, double vol, double hw0, double* val, double* err, int* split) {
  if constexpr (DIM == 1) {
    auto wg = [](int i) { return gk_wg(i); };
    auto wgk = [](int i) { return gk_wgk(i); };
    for (int k = 0; k < FDIM; ++k) {
      auto V = [&](int i) { return f[i * FDIM + k]; };
      double rg = V(0) * wg(3), rk = V(0) * wgk(7);
      double rabs = fabs(rk);
      int n = 1;
      for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        double v = V(n) + V(n + 1);
        rg += wg(j) * v;
        rk += wgk(j2) * v;
        rabs += wgk(j2) * (fabs(V(n)) + fabs(V(n + 1)));
        n += 2;
      }
      for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rk += wgk(j2) * (V(n) + V(n + 1));
        rabs += wgk(j2) * (fabs(V(n)) + fabs(V(n + 1)));
        n += 2;
      }
      val[k] = rk * hw0;
      double mean = rk * 0.5;
      double rasc = wgk(7) * fabs(V(0) - mean);
      n = 1;
      for (int j = 0; j < 3; ++j) {
        int j2 = 2 * j + 1;
        rasc += wgk(j2) * (fabs(V(n) - mean) + fabs(V(n + 1) - mean));
        n += 2;
      }
      for (int j = 0; j < 4; ++j) {
        int j2 = 2 * j;
        rasc += wgk(j2) * (fabs(V(n) - mean) + fabs(V(n + 1) - mean));
        n += 2;
      }
      double e = fabs(rk - rg) * hw0;
      rabs *= hw0;
      rasc *= hw0;
      if (rasc != 0 && e != 0) {
        double scale = pow(200 * e / rasc, 1.5);
        e = (scale < 1) ? rasc * scale : rasc;
      }
      const double dmin = 2.2250738585072014e-308, deps = 2.220446049250313e-16;
      if (rabs > dmin / (50 * deps)) {
        double me = 50 * deps * rabs;
        if (me > e) e = me;
      }
      err[k] = e;
    }
    *split = 0;
  } else {
    const double w1 = (double)(12824 - 9120 * DIM + 400 * DIM * DIM) / 19683.0;
    const double w3 = (double)(1820 - 400 * DIM) / 19683.0;
    const double w5 = 6859.0 / 19683.0 / (double)(1u << DIM);
    const double wE1 = (double)(729 - 950 * DIM + 50 * DIM * DIM) / 729.0;
    const double wE3 = (double)(265 - 100 * DIM) / 1458.0;
    const double w2 = 980. / 6561., w4 = 200. / 19683., wE2 = 245. / 486., wE4 = 25. / 729.;
    double diff[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) diff[d] = 0;
    for (int k = 0; k < FDIM; ++k) {
      auto V = [&](int i) { return f[i * FDIM + k]; };
      double val0 = V(0), s2 = 0, s3 = 0, s4 = 0, s5 = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double v0 = V(1 + 4 * d), v1 = V(2 + 4 * d), v2 = V(3 + 4 * d), v3 = V(4 + 4 * d);
        s2 += v0 + v1;
        s3 += v2 + v3;
        diff[d] += fabs(v0 + v1 - 2 * val0 - GM::ratio * (v2 + v3 - 2 * val0));
      }
      int k0 = 1 + 4 * DIM;
      for (int i = 0; i < 2 * DIM * (DIM - 1); ++i) s4 += V(k0 + i);
      k0 += 2 * DIM * (DIM - 1);
      for (int i = 0; i < (1 << DIM); ++i) s5 += V(k0 + i);
      double r7 = vol * (w1 * val0 + w2 * s2 + w3 * s3 + w4 * s4 + w5 * s5);
      double r5 = vol * (wE1 * val0 + wE2 * s2 + wE3 * s3 + wE4 * s4);
      val[k] = r7;
      err[k] = fabs(r5 - r7);
    }
    double md = 0;
    int dm = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
      if (diff[d] > md) {
        md = diff[d];
        dm = d;
      }
    *split = dm;
  }
}

// ---------------------------------------------------------------------------
// block-wide helpers
template <int NT>
__device__ inline double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = (l < NT / 32) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (l == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  return t;
}

template <int NT>
__device__ inline int block_exclusive_scan(int v, int* red, int* total) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (l >= o) x += y;
  }
  __syncthreads();
  if (l == 31) red[w] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    int t = (l < NT / 32) ? red[l] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (l >= o) t += y;
    }
    red[l + 32] = t;  // inclusive warp-prefix of warp totals
  }
  __syncthreads();
  int base = (w > 0) ? red[32 + w - 1] : 0;
  *total = red[32 + NT / 32 - 1];
  return base + x - v;
}

__device__ inline bool converged_check(int fdim, int norm, const double* V, const double* E, double abs_tol,
                                       double rel_tol) {
  if (fdim == 1 || norm == TP_NORM_INDIVIDUAL) {
    for (int k = 0; k < fdim; ++k)
      if (E[k] > abs_tol && E[k] > fabs(V[k]) * rel_tol) return false;
    return true;
  }
  // L1 (the only multi-component norm used on this path)
  double e = 0, v = 0;
  for (int k = 0; k < fdim; ++k) {
    e += E[k];
    v += fabs(V[k]);
  }
  return e <= abs_tol || e <= v * rel_tol;
}

// Shared scratch of the engine (besides the policy's own)
template <int FDIM>
struct EngineShared {
  int live_list[1024];  // live points of the current chunk
  int nlive_chunk;
  unsigned long long hist[256];
  double red[64];
  int ired[80];
  double V[FDIM], E[FDIM];
  unsigned long long q_above;
  unsigned long long prefix;
  int job, nlive, npend, status, stop, ktot, sweeps;
  long long neval;
};

// Dynamic shared memory of adaptive_body for policy P.
template <int DIM, int FDIM, class P>
__host__ __device__ constexpr size_t engine_smem_bytes() {
  return ((P::PSMEM + 15) & ~size_t(15)) + (((size_t)P::CH * GMRule<DIM>::NP * P::REC + 15) & ~size_t(15)) +
         sizeof(double) * (size_t)P::G * P::CH * GMRule<DIM>::NP * P::PD +
         sizeof(double) * (size_t)P::CH * GMRule<DIM>::NP * FDIM + sizeof(EngineShared<FDIM>) + 16;
}


// ---------------------------------------------------------------------------
// The persistent adaptive-integration kernel body. Policy P provides:
//   static constexpr int G, REC (bytes per point record), CH (regions/chunk)
//   __device__ void begin_job(int job, char* psmem, double* xmin, double* xmax) (all threads; syncs inside)
//   __device__ bool setup(int p, const double* x, char* rec)   (true: point needs its groups)
//   __device__ bool is_live(const char* rec)
//   __device__ void group(const char* rec, int g, double* part /*PD*/)  (live points only)
//   static int slot(int g): sum class of group g (0..NS-1)
//   __device__ void finalize(const char* rec, const double* sum /*FDIM*/, double* fval /*FDIM*/)
//   __device__ void end_job(int job, const double* V, const double* E, long long neval, int status)
//   static constexpr size_t PSMEM (policy shared bytes)
//
// CS > 1 (launch with thread-block clusters of CS CTAs): the CTAs of a
// cluster own one integral together. Every sweep's pending regions are dealt
// out to them in chunks (rank r takes chunks r, r + CS, ...); the region store
// is the cluster's, in HBM; rank 0 alone does the totals, the selection and
// the splitting, and publishes the job, the pending count and the stop flag
// in its shared memory, which the other ranks read through distributed shared
// memory. Two cluster barriers per sweep (after the evaluation, after the
// bookkeeping), with release/acquire ordering of the region store; every rank
// takes the same branches, decided from rank 0's published values after a
// barrier. The region sequence is that of CS = 1.
template <int CS>
__device__ __forceinline__ void engine_cluster_sync() {
  if constexpr (CS > 1) {
    __threadfence();
    cooperative_groups::this_cluster().sync();
  } else {
    __syncthreads();
  }
}

template <int DIM, int FDIM, int NT, class P, int CS = 1>
__device__ void adaptive_body(P& pol, int njobs, int* job_counter, const EngineCfg cfg, char* scratch,
                              size_t slot_bytes) {
  constexpr int NP = GMRule<DIM>::NP;
  constexpr int CH = P::CH;
  constexpr int G = P::G;
  constexpr int PD = P::PD;  // values per group item (>= 1)
  constexpr int NS = P::NS;  // group classes: item g adds into sum class P::slot(g)
  static_assert(P::CH * NP <= 1024, "live list holds one chunk");
  extern __shared__ __align__(16) char smem[];
  char* psmem = smem;
  char* recs = psmem + ((P::PSMEM + 15) & ~size_t(15));
  double* part = (double*)(recs + (((size_t)CH * NP * P::REC + 15) & ~size_t(15)));  // [G][CH*NP][PD]
  double* fval = part + (size_t)G * CH * NP * PD;                                 // [CH*NP][FDIM]
  EngineShared<FDIM>* es = (EngineShared<FDIM>*)(fval + (size_t)CH * NP * FDIM);
  // the control block every rank follows: rank 0's (distributed shared memory)
  EngineShared<FDIM>* es0 = es;
  int crank = 0;
  if constexpr (CS > 1) {
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    crank = (int)cl.block_rank();
    es0 = cl.map_shared_rank(es, 0);
  }

  Slot<DIM, FDIM> S;
  S.init(scratch + (size_t)(blockIdx.x / CS) * slot_bytes, cfg.cap);
  const int tid = threadIdx.x;

  for (;;) {
    if (crank == 0 && tid == 0) {
      int k = atomicAdd(job_counter, 1);
      es->job = (k < njobs && pol.job_order) ? pol.job_order[k] : k;
      es->ktot = k;
    }
    engine_cluster_sync<CS>();
    const int job = es0->job;
    if (es0->ktot >= njobs) break;
    double xmin[DIM], xmax[DIM];
    pol.begin_job(job, psmem, xmin, xmax);
    if (tid == 0) es->nlive_chunk = 0;
    if (crank == 0 && tid == 0) {
      for (int d = 0; d < DIM; ++d) {
        S.cen[(size_t)d * S.cap] = 0.5 * (xmin[d] + xmax[d]);
        S.hw[(size_t)d * S.cap] = 0.5 * (xmax[d] - xmin[d]);
      }
      double v = 1;
      for (int d = 0; d < DIM; ++d) v *= 2 * (0.5 * (xmax[d] - xmin[d]));
      S.vol[0] = v;
      S.pend[0] = 0;
      es->nlive = 1;
      es->npend = 1;
      es->status = 0;
      es->stop = 0;
      es->neval = 0;
      es->sweeps = 0;
    }
    engine_cluster_sync<CS>();

    for (int sweep = 0;; ++sweep) {
      // ---------------- evaluate the pending regions ----------------------
      const int npend = es0->npend;
      // a cluster deals out chunks of CH regions, or single regions while a
      // sweep has fewer than CS * CH of them (all ranks then have work)
      const int step = (CS > 1 && npend < CS * CH) ? 1 : CH;
      for (int base = crank * step; base < npend; base += CS * step) {
        const int nreg = min(step, npend - base);
        const int npts = nreg * NP;
        // (a) point setup; points that need the expensive inner sums are
        //     appended to a compact live list
        for (int p = tid; p < npts; p += NT) {
          int r = S.pend[base + p / NP];
          double c[DIM], h[DIM], x[DIM];
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            c[d] = S.cen[(size_t)d * S.cap + r];
            h[d] = S.hw[(size_t)d * S.cap + r];
          }
          rule_point<DIM>(p % NP, c, h, x);
          if (pol.setup(p, x, recs + (size_t)p * P::REC)) es->live_list[atomicAdd(&es->nlive_chunk, 1)] = p;
        }
        __syncthreads();
        // (b) (live point, group) items: equal-cost work for every thread
        const int nl = es->nlive_chunk;
        for (int it = tid; it < nl * G; it += NT) {
          int g = it / nl, q = it - g * nl;
          int p = es->live_list[q];
          double pv[PD];
          pol.group(recs + (size_t)p * P::REC, g, pv);
#pragma unroll
          for (int k = 0; k < PD; ++k) part[((size_t)g * npts + p) * PD + k] = pv[k];
        }
        __syncthreads();
        // (c) per-point totals (fixed group order -> deterministic)
        for (int p = tid; p < npts; p += NT) {
          double s[NS * PD];
#pragma unroll
          for (int k = 0; k < NS * PD; ++k) s[k] = 0;
          if (pol.is_live(recs + (size_t)p * P::REC))
            for (int g = 0; g < G; ++g) {
              const int sl = P::slot(g);
#pragma unroll
              for (int k = 0; k < PD; ++k) s[sl * PD + k] += part[((size_t)g * npts + p) * PD + k];
            }
          pol.finalize(recs + (size_t)p * P::REC, s, fval + (size_t)p * FDIM);
        }
        if (tid == 0) es->nlive_chunk = 0;
        __syncthreads();
        for (int rr = tid; rr < nreg; rr += NT) {
          int r = S.pend[base + rr];
          double v[FDIM], e[FDIM];
          int sp;
          rule_combine<DIM, FDIM>(fval + (size_t)rr * NP * FDIM, S.vol[r], S.hw[r], v, e, &sp);
          double em = 0;
#pragma unroll
          for (int k = 0; k < FDIM; ++k) {
            S.val[(size_t)k * S.cap + r] = v[k];
            S.err[(size_t)k * S.cap + r] = e[k];
            em = fmax(em, e[k]);
          }
          S.emax[r] = em;
          S.split[r] = (uint8_t)sp;
        }
        __syncthreads();
      }
      if constexpr (CS > 1) engine_cluster_sync<CS>();
      // rank 0: totals, convergence, selection and splitting; a stop sets
      // es->stop and leaves this block
      if (crank == 0) do {
      if (tid == 0) es->neval += (long long)npend * NP;

      // ---------------- totals and convergence ----------------------------
      const int nlive = es->nlive;
      double tv[FDIM], te[FDIM];
#pragma unroll
      for (int k = 0; k < FDIM; ++k) {
        double a = 0, b = 0;
        for (int i = tid; i < nlive; i += NT) {
          a += S.val[(size_t)k * S.cap + i];
          b += S.err[(size_t)k * S.cap + i];
        }
        tv[k] = block_sum<NT>(a, es->red);
        te[k] = block_sum<NT>(b, es->red);
      }
      bool conv = converged_check(FDIM, cfg.norm, tv, te, cfg.abs_tol, cfg.rel_tol);
      if (conv || sweep + 1 >= cfg.max_sweeps) {
        if (tid == 0) {
          for (int k = 0; k < FDIM; ++k) {
            es->V[k] = tv[k];
            es->E[k] = te[k];
          }
          if (!conv) es->status |= 2;
          es->sweeps = sweep + 1;
          es->stop = 1;
        }
        __syncthreads();
        break;
      }
      // tolerance for the Gladwell pop loop
      double etot = 0, vabs = 0;
      bool l1 = !(FDIM == 1 || cfg.norm == TP_NORM_INDIVIDUAL);
#pragma unroll
      for (int k = 0; k < FDIM; ++k) {
        etot += te[k];
        vabs += fabs(tv[k]);
      }
      double tol;
      if (l1)
        tol = fmax(cfg.abs_tol, vabs * cfg.rel_tol);
      else
        tol = fmax(cfg.abs_tol, fabs(tv[0]) * cfg.rel_tol);

      // ---------------- radix select of the error threshold ---------------
      // Errors are summed as 62-bit fixed-point fractions of the total error,
      // so the histogram sums (shared-memory integer atomics) are exact and
      // independent of the order of the additions.
      const double qscale = 4.611686018427387904e18 / etot;  // 2^62 / E_tot
      const double tol_q = tol * qscale;
      if (tid == 0) {
        es->prefix = 0ull;
        es->q_above = 0ull;
      }
      for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (int b = tid; b < 256; b += NT) es->hist[b] = 0ull;
        __syncthreads();
        const unsigned long long pre = es->prefix;
        for (int i = tid; i < nlive; i += NT) {
          unsigned long long key = (unsigned long long)__double_as_longlong(S.emax[i]);
          if (pass == 0 || (key >> (shift + 8)) == pre) {
            double es_ = 0;
#pragma unroll
            for (int k = 0; k < FDIM; ++k) es_ += S.err[(size_t)k * S.cap + i];
            atomicAdd(&es->hist[(key >> shift) & 255ull], (unsigned long long)(es_ * qscale));
          }
        }
        __syncthreads();
        if (tid < 32) {
          const int l = tid;
          unsigned long long loc[8];
          unsigned long long ls = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            loc[q] = es->hist[8 * l + q];
            ls += loc[q];
          }
          // pass 0 histograms every region: its sum is the fixed-point total
          unsigned long long tot = ls;
          for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
          __shared__ unsigned long long s_qtot;
          if (pass == 0 && l == 0) s_qtot = tot;
          __syncwarp();
          const unsigned long long qtot = s_qtot;
          // suffix sum over lanes (lane l: sum of lanes > l)
          unsigned long long suf = ls;
          for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_down_sync(0xffffffffu, suf, o);
            if (l + o < 32) suf += y;
          }
          unsigned long long cum = es->q_above + (suf - ls);
          int best = -1;
          unsigned long long cum_best = 0;
#pragma unroll
          for (int q = 7; q >= 0; --q) {
            cum += loc[q];
            if (best < 0 && (double)(qtot > cum ? qtot - cum : 0ull) <= tol_q) {
              best = 8 * l + q;
              cum_best = cum;
            }
          }
          int chosen = __reduce_max_sync(0xffffffffu, best);
          bool none = chosen < 0;
          if (none) chosen = 0;
          unsigned long long cb = (best == chosen && !none) ? cum_best : 0ull;
          unsigned long long hb = (best == chosen && !none) ? es->hist[chosen] : 0ull;
          for (int o = 16; o > 0; o >>= 1) {
            cb += __shfl_xor_sync(0xffffffffu, cb, o);
            hb += __shfl_xor_sync(0xffffffffu, hb, o);
          }
          unsigned long long all = ls;
          for (int o = 16; o > 0; o >>= 1) all += __shfl_xor_sync(0xffffffffu, all, o);
          if (l == 0) {
            // bins strictly above the chosen one are selected for sure; when no
            // bin satisfies the tolerance (rounding), take the whole range
            es->q_above = none ? es->q_above + all - es->hist[0] : cb - hb;
            es->prefix = (pre << 8) | (unsigned long long)chosen;
          }
        }
        __syncthreads();
      }
      const unsigned long long tau = es->prefix;

      // ---------------- compaction: split every region with key >= tau ----
      const int chunk = (nlive + NT - 1) / NT;
      const int lo = min(tid * chunk, nlive), hi = min(lo + chunk, nlive);
      int cnt = 0;
      for (int i = lo; i < hi; ++i)
        cnt += ((unsigned long long)__double_as_longlong(S.emax[i]) >= tau) ? 1 : 0;
      int ktot;
      int rank = block_exclusive_scan<NT>(cnt, es->ired, &ktot);
      if (ktot == 0 || nlive + ktot > S.cap) {
        if (tid == 0) {
          for (int k = 0; k < FDIM; ++k) {
            es->V[k] = tv[k];
            es->E[k] = te[k];
          }
          es->status |= (ktot == 0) ? 4 : 1;
          es->sweeps = sweep + 1;
          es->stop = 1;
        }
        __syncthreads();
        break;
      }
      for (int i = lo; i < hi; ++i) {
        if ((unsigned long long)__double_as_longlong(S.emax[i]) < tau) continue;
        const int u = nlive + rank;
        const int d = S.split[i];
        double v = 1;
#pragma unroll
        for (int q = 0; q < DIM; ++q) {
          double cq = S.cen[(size_t)q * S.cap + i];
          double hq = S.hw[(size_t)q * S.cap + i];
          if (q == d) {
            hq *= 0.5;
            S.cen[(size_t)q * S.cap + i] = cq - hq;
            S.hw[(size_t)q * S.cap + i] = hq;
            S.cen[(size_t)q * S.cap + u] = cq + hq;
          } else {
            S.cen[(size_t)q * S.cap + u] = cq;
          }
          S.hw[(size_t)q * S.cap + u] = hq;
          v *= 2 * hq;
        }
        S.vol[i] *= 0.5;
        S.vol[u] = v;
        S.pend[2 * rank] = i;
        S.pend[2 * rank + 1] = u;
        ++rank;
      }
      __syncthreads();
      if (tid == 0) {
        es->nlive = nlive + ktot;
        es->npend = 2 * ktot;
      }
      } while (0);
      engine_cluster_sync<CS>();
      if (es0->stop) break;
    }
    if (crank == 0) pol.end_job(job, es->V, es->E, es->neval, es->status);
    __syncthreads();
  }
  // no rank leaves while another may still read rank 0's shared memory
  if constexpr (CS > 1) cooperative_groups::this_cluster().sync();
}


}  // namespace tp
