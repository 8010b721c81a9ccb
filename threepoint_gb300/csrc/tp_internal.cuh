// Internal declarations shared by the CUDA translation units of
// libthreepoint_gb300.so. Nothing here is part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/threepoint_gb300.h"

namespace tp {

constexpr int NZ = 256;          // redshift bins of the tables (n_redshift_bins)
constexpr int NK = 256;          // k bins of a tabulated linear P(k) (n_kbins)
constexpr int NNODE = 96;        // Gauss-Legendre nodes of every line-of-sight integral
constexpr double EPS = 1.0e-4;   // accuracy of the sigma(R)/growth iterations
constexpr double H0_OVER_C = 100. / 299792.;
constexpr double C_OVER_H0 = 2997.92;
constexpr double PI = 3.14159265358979323846;
constexpr double LOG2_10 = 3.32192809488736234787;
constexpr double LN2 = 0.69314718055994530942;
// FP32 integrands read the Eisenstein & Hu linear P(k) from a per-cosmology
// table of log2 P on a uniform log2(k h) grid, interpolated by Catmull-Rom
// cubics (relative error ~1e-6 over the grid); FP64 integrands evaluate the
// fit itself.
constexpr int PLT_N = 1024;  // grid points; the table stores per interval (y0, c1, c2, c3) of the cubic
constexpr double PLT_LO = -24.0, PLT_HI = 24.0;
// 2 ln T(k) of the Eisenstein & Hu no-wiggle transfer function, the part of
// the sigma(R) integrand that does not depend on R, on the grid
// t_i = EHG_T0 + i / EHG_PER_UNIT in t = ln(k h^-1 Mpc), i < EHG_N (ln k in
// [-16, 12]); 4-point Lagrange interpolation is within 3e-13 of the formula
constexpr int EHG_N = 28704;
constexpr double EHG_T0 = -16.0, EHG_PER_UNIT = 1024.0;

// Per-cosmology parameter block as uploaded to the device.
struct CosmoDev {
  double h, sigma8, omb, omc, ns, w, om, ow, zmax;
  int pk_given;
  double dk, kmin, kmax;
  double sigma_eps, ngal;  // shape noise for the power spectrum (covariance)
  int constant_ps;
};

// Eisenstein & Hu no-wiggle constants hoisted out of linear_pk
// (the cosmology-only part of cuda_version/bispectrum.cu:651-680).
struct EHConst {
  double h, omh2, theta2, sa, one_m_sa, sh, c184, ehc, ns;
};

// FP64 z-tables of one cosmology (set_cosmology output), row layout
// [f_K, g, D1, r_sigma, n_eff, ncur] x 256, then norm and dz.
struct TablesDev {
  double f_K[NZ], g[NZ], D1[NZ], r_sigma[NZ], n_eff[NZ], ncur[NZ];
  double pk[NK];
  double norm, dz;
  double lgr0;  // growth integral at z = 0 (D1 = lgr(z) / lgr0)
};

// Per-node BiHalofit coefficients for the fixed line-of-sight nodes of
// b_kappa: everything in bispec() that depends on z only, precomputed once
// per cosmology. Stored structure-of-arrays: coef[c * NNODE + node].
enum NodeCoef {
  NC_W = 0,    // LOS weight: gauss w * dz/2 * 27/8 Om^3 (H0/c)^5 * (g(1+z))^3 / f_K / E
  NC_S,        // r_sigma / f_K            (q = ell * S)
  NC_L2S,      // log2(r_sigma / f_K)
  NC_HF,       // h / f_K                  (k[1/Mpc] = ell * HF)
  NC_L2HF,     // log2(h / f_K)
  NC_ANA,      // log2(10) * (-2.167 - 2.944 ls - 1.106 ls^2 - 2.865 ls^3)
  NC_ANR,      // 0.310 * log2(10)
  NC_ANC,      // 10^(0.182 + 0.57 n_eff)
  NC_BN, NC_CN,
  NC_ALA,      // log2(10) * (-4.348 - 3.006 n - 0.5745 n^2)
  NC_ALD,      // log2(10) * 10^(-0.9 + 0.2 n)
  NC_BETAB,    // 10^(-1.731 - 2.845 n - 1.4995 n^2 - 0.2811 n^3)
  NC_FN, NC_GN, NC_HN, NC_MN, NC_NN, NC_MUN, NC_NUN, NC_PN, NC_EN,
  NC_DN,       // 10^(-0.483 + 0.892 ls - 0.086 Om(z)) (F2 correction)
  NC_D1SQ,     // D1^2
  NC_TREE,     // 1 when z > 10 (tree-level bispectrum), else 0
  NC_D1P4,     // D1^4 (tree level)
  NC_COUNT
};
// node tables are stored node-major with this pitch (16-byte rows for float4 loads)
constexpr int NCP = 28;
static_assert(NC_COUNT <= NCP, "node coefficient pitch");

// FP32 node rows of the <Map^3> / b_kappa point path: the same BiHalofit
// coefficients with every product that does not involve the triangle folded
// in (q_i = ell_i s enters only through s-scaled coefficients; multiplicative
// factors of powers are added to their log2 exponents), so that one
// (point, node) evaluation needs fewer instructions. Same pitch and node-major
// layout as the NC_* rows.
enum FastCoef {
  NF_W = 0,     // NC_W / wscale
  NF_L2S,       // log2(s), s = r_sigma / f_K        (log2 q_i = lg_i + NF_L2S)
  NF_L2HF,      // log2(h / f_K)
  NF_HF,        // h / f_K
  NF_TOFF,      // (NF_L2HF - PLT_LO) * (PLT_N-1)/(PLT_HI-PLT_LO): P_lin table coordinate offset
  NF_ANA,       // log2 a_n = NF_ANA - ex2(NF_ANC log2 r1 + NF_L2ANR)
  NF_L2ANR,     // log2(0.310 log2(10))
  NF_ANC,
  NF_L2BN,      // log2 b_n
  NF_CNS,       // c_n s
  NF_ALA, NF_ALD, NF_BETAB,
  NF_D1SQ,      // D1^2
  NF_D1SQFNS2,  // D1^2 f_n s^2
  NF_GNS,       // g_n s
  NF_HNS2,      // h_n s^2
  NF_L2MN, NF_L2NN,  // log2 m_n, log2 n_n
  NF_MUN, NF_NUN,
  NF_PNS,       // p_n s
  NF_ENS,       // e_n s
  NF_DNS,       // d_n s
  NF_TREE,      // 1 when z > 10
  NF_D1P4,      // D1^4
  NF_COUNT
};
static_assert(NF_COUNT <= NCP, "fast node coefficient pitch");

// Per-node Halofit coefficients for the P_kappa line-of-sight integral
// (P_k_nonlinear + limber prefactor at the fixed nodes; z-only parts).
enum HaloCoef {
  HC_W = 0,    // gauss w * dz/2 * 9/4 (H0/c)^3 Om^2 (1+z)^2 g^2 / E   (0 below z=1e-5)
  HC_INVFK,    // 1/f_K
  HC_RS,       // r_sigma
  HC_D1SQ,     // D1^2
  HC_A, HC_B, HC_C, HC_GAM, HC_ALPHA, HC_BETA, HC_XNU,
  HC_F1, HC_F2, HC_F3,
  HC_L2INVFK,  // log2(1/f_K)
  HC_L2RS,     // log2(r_sigma)
  HC_L2F3C,    // log2(f3 * c)
  HC_COUNT
};

// Halo model of the covariance terms T5, T6, T7 (cuda_version/halomodel.cu).
constexpr int NM = 128;                          // mass bins of the sigma^2(m) tables (n_mbins)
constexpr double LOGM_MIN = 9.0, LOGM_MAX = 17.0;  // log10(M / (Msun/h)) range
constexpr double RHO_CRIT = 2.7754e11;           // critical density [Msun h^2 / Mpc^3]

// Per-node rows of the halo-model line-of-sight integrals (z-only parts of
// trispectrum_integrand / pentaspectrum_integrand at the 96 fixed nodes, in
// the node order of the other node tables). The halo model reads f_K, g and
// D1 by linear interpolation on the grid z_i = i z_max / 255
// (halomodel.cu:300-311,398-408), not by the mid-bin rule of b_kappa.
enum HaloNodeRow {
  HN_INVCHI = 0,  // 1 / f_K(z)
  HN_D1SQ,        // D1(z)^2
  HN_DC2,         // delta_c(z)^2, delta_c = 1.686 (1 + 0.0123 log10 Om(z))
  HN_CZ,          // (1 + z)^-1.01 (redshift part of the Duffy et al. concentration)
  HN_WTRI,        // gauss w dz/2 g^4 / f_K^2 (c/H0) / E (1.5 Om (H0/c)^2)^4 (1+z)^4
  HN_WPEN,        // gauss w dz/2 g^6 / f_K^4 (c/H0) / E (1.5 Om (H0/c)^2)^6 (1+z)^6
  HN_COUNT
};

// Halo-model tables of one cosmology: sigma^2(m_i) and dsigma^2/dm(m_i) at
// z = 0 for m_i = 10^(LOGM_MIN + i (LOGM_MAX - LOGM_MIN) / NM), and the node rows.
// hnf holds the same rows in FP32 with the two weight rows divided by their
// largest node value, wmax[0] (HN_WTRI) and wmax[1] (HN_WPEN).
struct HaloTab {
  double sig2[NM], dsig2[NM];
  double hn[HN_COUNT * NNODE];
  float hnf[HN_COUNT * NNODE];
  double wmax[2];
};

// ---- helpers shared by several translation units ---------------------------
__host__ __device__ inline double eh_linear_pk(const EHConst& e, double k) {
  double kk = k * e.h;
  double x = 0.43 * kk * e.sh;
  double x2 = x * x;
  double geff = e.omh2 * (e.sa + e.one_m_sa / (1.0 + x2 * x2));
  double qeff = kk / geff * e.theta2;
  double L = log(2.718281828 + e.c184 * qeff);
  double C = 14.4 + 325.0 / (1.0 + 60.5 * pow(qeff, 1.11));
  double r = L / (L + C * qeff * qeff);
  return e.ehc * pow(kk, e.ns) * r * r;
}

EHConst make_eh_const(const CosmoDev& c, double norm);

// host-side 96-point Gauss-Legendre rule on [-1,1] (positive half, ascending)
void gauss_legendre96(double* a48, double* w48);

}  // namespace tp
