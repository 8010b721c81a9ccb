// Shared pieces of the command-line drivers: reading the cosmology and n(z)
// and building a one-cosmology context, as the reference drivers do with
// cosmology(fn), read_n_of_z and set_cosmology (cuda_version/cosmology.cu:11,
// helpers.cu:9, bispectrum.cu:100).
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "threepoint_gb300.h"

namespace cli {

[[noreturn]] inline void die(const std::string& what, int code = 1) {
  std::cerr << what << std::endl;
  exit(code);
}

inline void check(int st, const std::string& what, const tp_ctx* ctx = nullptr) {
  if (st == TP_OK) return;
  std::string msg = what + ": " + tp_status_string(st);
  if (ctx && tp_last_error(ctx)[0]) msg += " (" + std::string(tp_last_error(ctx)) + ")";
  die(msg);
}

// precision selected by an optional trailing "fp32" argument (FP64 otherwise)
inline int precision_arg(int argc, char** argv, int first_optional) {
  for (int i = first_optional; i < argc; ++i)
    if (std::string(argv[i]) == "fp32") return TP_FP32;
  return TP_FP64;
}

inline std::ostream& operator<<(std::ostream& o, const tp_cosmology& c) {
  // the parameter-file layout, as the reference's operator<< (cosmology.cu:80-90)
  o << "h " << c.h << std::endl
    << "sigma_8 " << c.sigma8 << std::endl
    << "Omega_b " << c.omb << std::endl
    << "n_s " << c.ns << std::endl
    << "w " << c.w << std::endl
    << "Omega_m " << c.om << std::endl
    << "z_max " << c.zmax << std::endl;
  return o;
}

// cosmology file + n(z) file -> context with that single cosmology (linear
// P(k) from the Eisenstein & Hu fit, as set_cosmology(cosmo, &nz) does)
inline tp_ctx* make_context(const std::string& cosmo_file, const std::string& nz_file, int device,
                            tp_cosmology* cosmo_out) {
  tp_cosmology c;
  check(tp_cosmology_from_file(cosmo_file.c_str(), &c), "reading cosmology " + cosmo_file);
  std::vector<double> nz(256);
  check(tp_read_n_of_z(nz_file.c_str(), 256, c.zmax, nz.data()), "reading n(z) " + nz_file);
  tp_ctx* ctx = nullptr;
  check(tp_ctx_create(device, &ctx), "creating the CUDA context");
  check(tp_set_cosmologies(ctx, &c, 1, nz.data(), 0, nullptr, 0, 0, 0), "building the cosmology tables", ctx);
  if (cosmo_out) *cosmo_out = c;
  return ctx;
}

// convert_rad_to_angle (helpers.cu:155-174): factors 3437.74677 (arcmin), 57.3 (deg)
inline double rad_to_arcmin(double v) { return 3437.74677 * v; }
inline double rad_to_deg(double v) { return 57.3 * v; }

}  // namespace cli
