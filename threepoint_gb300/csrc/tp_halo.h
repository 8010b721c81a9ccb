// Halo-model covariance terms T5, T6, T7 (tp_halo.cu).
#pragma once
#include <array>
#include <vector>

#include "tp_capi_internal.h"

namespace tp {

// host lower bound of the T5/T6/T7 ell integrals (the reference sets its
// host lMin to 1e-4 there, apertureStatisticsCovariance.cu:1206,1244,1287)
constexpr double HALO_LMIN = 1e-4;

// upper ell bound of term 5, 6 or 7 for the radii t[0..5]: 10 / the larger
// (T5, T6) or smaller (T7) of the two triplets' smallest radii
double halo_lmax(int term, const double* t);

// Builds the halo-model tables (sigma^2(m), dsigma^2/dm, node rows) of a
// cosmology on first use.
int ensure_halo(tp_ctx* ctx, int cosmo);

// The halo integral of T5, T6 or T7 for each radius set th6[i] (T6 without
// its 1-D ell_1 factor), normalised as the reference normalises them;
// precision TP_FP64 or TP_FP32 (node arithmetic; the cubature is FP64).
int halo_terms(tp_ctx* ctx, int cosmo, int term, int geom, double theta_max, double area,
               const std::vector<std::array<double, 6>>& th6, int precision, std::vector<double>& out, int& bad);

}  // namespace tp
