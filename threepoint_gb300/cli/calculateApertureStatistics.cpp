// calculateApertureStatistics.x -- <Map^3> for all theta1 <= theta2 <= theta3 of
// a list of aperture radii; same arguments and output file as the reference
// driver (cuda_version/calculateApertureStatistics.cu:19-133). All triplets go
// to the GPU in one batch instead of one MapMapMap call each.
//
//   calculateApertureStatistics.x cosmo.dat thetas.dat out.dat nz.dat [fp32]
//
// Output: one line "theta1 theta2 theta3 <Map^3> " per triplet, radii in arcmin
// as read from the thetas file.
#include <fstream>

#include "cli_common.hpp"

static const char* kUsage = R"(
calculateApertureStatistics.x : Wrong number of command line parameters (Needed: 5)
Argument 1: Filename for cosmological parameters (ASCII, see necessary_files/MR_cosmo.dat for an example)
Argument 2: Filename with thetas [arcmin]
Argument 3: Outputfilename, directory needs to exist
Argument 4: Filename for n(z) (ASCII, see necessary_files/nz_MR.dat for an example)
Argument 5 (optional, not in the reference): fp32 to evaluate the FP32 integrand

Example:
./calculateApertureStatistics.x ../necessary_files/MR_cosmo.dat ../necessary_files/HOWLS_thetas.dat ../../results_MR/MapMapMap_bispec_gpu_nz.dat ../necessary_files/nz_MR.dat
)";

int main(int argc, char* argv[]) {
  if (argc < 5) cli::die(kUsage);
  const std::string cosmo_file = argv[1], thetas_file = argv[2], out_file = argv[3], nz_file = argv[4];
  const int precision = cli::precision_arg(argc, argv, 5);

  std::ofstream out(out_file);
  if (!out.is_open()) cli::die("Couldn't open " + out_file);

  std::vector<double> thetas(4096);
  int n = 0;
  cli::check(tp_read_thetas(thetas_file.c_str(), thetas.data(), (int)thetas.size(), &n), "reading " + thetas_file);
  if (n > (int)thetas.size()) cli::die("too many aperture radii in " + thetas_file);
  thetas.resize(n);

  tp_cosmology cosmo;
  tp_ctx* ctx = cli::make_context(cosmo_file, nz_file, 0, &cosmo);
  std::cerr << "Using cosmology from " << cosmo_file << ":" << std::endl;
  cli::operator<<(std::cerr, cosmo);
  std::cerr << "Using thetas in " << thetas_file << std::endl;
  std::cerr << "Writing to:" << out_file << std::endl;
  std::cerr << "Using n(z) from " << nz_file << std::endl;

  // triplets theta1 <= theta2 <= theta3 in the reference's loop order (:87-110)
  std::vector<double> th_rad;
  std::vector<int> idx;
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++)
      for (int k = j; k < n; k++) {
        for (int t : {i, j, k}) {
          double r;
          cli::check(tp_convert_angle_to_rad(thetas[t], "arcmin", &r), "converting radii");
          th_rad.push_back(r);
          idx.push_back(t);
        }
      }
  const int ntrip = (int)(th_rad.size() / 3);
  std::vector<double> map3(ntrip);
  std::vector<int> status(ntrip);
  int st = tp_map3_batch(ctx, nullptr, 1, th_rad.data(), ntrip, 0.0, 2 * M_PI, 1.0, 0.0, 1e-4, precision,
                         map3.data(), nullptr, nullptr, status.data());
  if (st == TP_ERR_CAPACITY)
    std::cerr << "warning: " << tp_last_error(ctx) << std::endl;
  else
    cli::check(st, "<Map^3>", ctx);

  for (int t = 0; t < ntrip; ++t)  // output loop of the reference (:118-130)
    out << thetas[idx[3 * t]] << " " << thetas[idx[3 * t + 1]] << " " << thetas[idx[3 * t + 2]] << " " << map3[t]
        << " " << std::endl;
  std::cerr << ntrip << " <Map^3> values written" << std::endl;
  tp_ctx_destroy(ctx);
  return 0;
}
