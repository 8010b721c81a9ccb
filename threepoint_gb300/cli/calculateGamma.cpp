// calculateGamma.x -- natural components Gamma^0..Gamma^3 of the shear 3PCF on
// the (r, u, v) binning of a config file; same arguments and output file as
// the reference driver (cuda_version/calculateGamma.cu:21-152). All triangles
// go to the GPU in one batch.
//
//   calculateGamma.x cosmo.dat gamma_config.dat out.dat nz.dat [device] [fp32]
//
// Output: one line "Re G0 Im G0 Re G1 Im G1 Re G2 Im G2 Re G3 Im G3 r u v" per
// bin centre, r-major then u then v.
#include <cmath>
#include <fstream>

#include "cli_common.hpp"

static const char* kUsage = R"(
calculateGamma.x : Wrong number of command line parameters (Needed: 4)
Argument 1: Filename for cosmological parameters (ASCII, see necessary_files/MR_cosmo.dat for an example)
Argument 2: Config file for the 3pcf
Argument 3: Outputfilename, directory needs to exist
Argument 4: Filename for n(z) (ASCII, see necessary_files/nz_MR.dat for an example)
Argument 5 (optional): GPU device number
Argument 6 (optional, not in the reference): fp32 to evaluate the FP32 integrand
Example:
./calculateGamma.x ../necessary_files/MR_cosmo.dat ../../results_MR/MapMapMap_varyingCosmos.dat ../necessary_files/nz_MR.dat 0
)";

int main(int argc, char** argv) {
  if (argc < 5) cli::die(kUsage);
  const std::string cosmo_file = argv[1], config_file = argv[2], out_file = argv[3], nz_file = argv[4];
  int device = 0;
  std::cout << "Executing " << argv[0] << " ";
  if (argc >= 6 && std::string(argv[5]) != "fp32") {
    device = atoi(argv[5]);
    std::cout << "on GPU " << device << std::endl;
  } else {
    std::cout << "on default GPU" << std::endl;
  }
  const int precision = cli::precision_arg(argc, argv, 5);

  tp_gamma_config cfg;
  cli::check(tp_gamma_config_from_file(config_file.c_str(), &cfg), "reading " + config_file);
  std::ofstream out(out_file);
  if (!out.is_open()) cli::die("Couldn't open " + out_file);

  tp_cosmology cosmo;
  tp_ctx* ctx = cli::make_context(cosmo_file, nz_file, device, &cosmo);
  std::cerr << "Using cosmology:" << std::endl;
  cli::operator<<(std::cerr, cosmo);
  std::cerr << "Writing to:" << out_file << std::endl;
  std::cerr << "Binning r in " << cfg.rsteps << " bins from " << cfg.rmin << " to " << cfg.rmax << std::endl;
  std::cerr << "Binning u in " << cfg.usteps << " bins from " << cfg.umin << " to " << cfg.umax << std::endl;
  std::cerr << "Binning v in " << cfg.vsteps << " bins from " << cfg.vmin << " to " << cfg.vmax << std::endl;
  std::cerr << "Setting the triangle center as Centroid" << std::endl;

  const long n = (long)cfg.rsteps * cfg.usteps * cfg.vsteps;
  std::vector<double> x(3 * n), ruv(3 * n);
  cli::check(tp_gamma_triangles(&cfg, x.data(), ruv.data()), "binning");
  std::vector<double> g(8 * n);
  std::vector<int> status(4 * n);
  int st = tp_gamma_batch(ctx, 0, x.data(), (int)n, 0xF, 1e-3, precision, g.data(), status.data());
  if (st == TP_ERR_CAPACITY)
    std::cerr << "warning: " << tp_last_error(ctx) << std::endl;
  else
    cli::check(st, "Gamma", ctx);

  for (long i = 0; i < n; ++i) {  // output of the reference (:138-149)
    const double* v = &g[8 * i];
    out << v[0] << " " << v[1] << " " << v[2] << " " << v[3] << " " << v[4] << " " << v[5] << " " << v[6] << " "
        << v[7] << " " << ruv[3 * i] << " " << ruv[3 * i + 1] << " " << ruv[3 * i + 2] << std::endl;
  }
  std::cerr << n << " triangles written" << std::endl;
  tp_ctx_destroy(ctx);
  return 0;
}
