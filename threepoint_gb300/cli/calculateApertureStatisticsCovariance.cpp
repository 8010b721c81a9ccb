// calculateApertureStatisticsCovariance.x -- covariance terms of <Map^3> for all
// pairs of theta triplets; same 13 arguments and output files as the reference
// driver (cuda_version/calculateApertureStatisticsCovariance.cu:21-387). Each
// requested term is one GPU batch over all pairs.
//
//   calculateApertureStatisticsCovariance.x cosmo.dat thetas.dat nz.dat outfolder/ cov_param.dat
//       T1 T2 T4 T5 T6 T7 T7_2h circle|square|infinite|rectangular [fp32]
//
// T5, T6 and T7 are the halo-model terms (FP64 whatever the precision
// argument). T7_2h is identically zero in the reference: its integrand
// (pentaspectrum_integrand_ssc, halomodel.cu:469-496) multiplies by the survey
// variance table dev_sigma2_from_windowfunction_array, which nothing in the
// reference fills (zero-initialised constant memory,
// apertureStatisticsCovariance.cu:28), so its hcubature_v returns 0 after the
// first region; this driver writes those zeros for the square and infinite
// geometries and fails for the others, as the reference throws there
// (:1340-1353). Output per term:
// outfolder + cov_<geometry>_term<k>Numerical_sigma_<s>_n_<n>_thetaMax_<t>_gpu.dat
// (T7_2h: ..._term7_2h_Numerical_...), an N x N symmetric matrix, one row per
// line, each value followed by a space.
#include <cstring>
#include <fstream>
#include <stdexcept>

#include "cli_common.hpp"

static const char* kUsage = R"(
calculateApertureStatisticsCovariance.x : Wrong number of command line parameters (Needed: 10)
Argument 1: Filename for cosmological parameters (ASCII, see necessary_files/MR_cosmo.dat for an example)
Argument 2: Filename with thetas [arcmin]
Argument 3: Filename with n(z)
Argument 4: Outputfolder (needs to exist)
Argument 5: Filename for covariance parameters (ASCII, see necessary_files/cov_param for an example)
Argument 6: Calculate T1? (0 or 1)
Argument 7: Calculate T2? (0 or 1)
Argument 8: Calculate T4? (0 or 1)
Argument 9: Calculate T5? (0 or 1)
Argument 10: Calculate T6? (0 or 1)
Argument 11: Calculate T7? (0 or 1)
Argument 12: Calculate T7_2H? (0 or 1)
Argument 13: Survey geometry, either circle, square, infinite, or rectangular
Argument 14 (optional, not in the reference): fp32 to evaluate the FP32 integrands
)";

// writeCov (apertureStatisticsCovariance.cu:47-92): upper triangle (row-major,
// j >= i) -> full symmetric N x N text matrix
static bool write_cov(const std::vector<double>& values, int n, const std::string& filename) {
  if ((long)values.size() != (long)n * (n + 1) / 2) throw std::out_of_range("writeCov: Values has wrong length");
  std::ofstream out(filename);
  if (!out.is_open()) return false;
  std::vector<double> m((size_t)n * n);
  size_t ix = 0;
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++) m[(size_t)i * n + j] = values[ix++];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++) m[(size_t)i * n + j] = m[(size_t)j * n + i];
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) out << m[(size_t)i * n + j] << " ";
    out << std::endl;
  }
  return true;
}

int main(int argc, char* argv[]) {
  if (argc != 14 && !(argc == 15 && std::string(argv[14]) == "fp32")) cli::die(kUsage, -1);
  const std::string cosmo_file = argv[1], thetas_file = argv[2], nz_file = argv[3], out_folder = argv[4],
                    cov_file = argv[5], type_str = argv[13];
  int calc[7];
  for (int i = 0; i < 7; ++i) calc[i] = std::stoi(argv[6 + i]) != 0;
  const char* names[7] = {"term1", "term2", "term4", "term5", "term6", "term7", "term7 (2h)"};
  for (int i = 0; i < 7; ++i) std::cerr << "Calculating " << names[i] << ":" << calc[i] << std::endl;
  const int precision = argc == 15 ? TP_FP32 : TP_FP64;

  std::cerr << "Using cosmology from " << cosmo_file << std::endl;
  std::cerr << "Using thetas from " << thetas_file << std::endl;
  std::cerr << "Using n(z) from " << nz_file << std::endl;
  std::cerr << "Results are written to " << out_folder << std::endl;
  std::cerr << "Using covariance parameters from" << cov_file << std::endl;

  tp_cov_params par;
  cli::check(tp_cov_params_from_file(cov_file.c_str(), &par), "reading " + cov_file);
  if (par.shapenoise_only) std::cerr << "WARNING: Uses constant powerspectrum" << std::endl;

  int geom;  // (:111-130)
  if (type_str == "circle") geom = TP_GEOM_CIRCLE;
  else if (type_str == "square") geom = TP_GEOM_SQUARE;
  else if (type_str == "infinite") geom = TP_GEOM_INFINITE;
  else if (type_str == "rectangular") geom = TP_GEOM_RECTANGLE;
  else cli::die("Cov type not correctly specified", -1);
  std::cerr << "Using survey geometry " << type_str << std::endl;
  // terms coded for some geometries only: the reference throws at the first
  // pair, before any output is written (apertureStatisticsCovariance.cu:1193,
  // 1227, 1237, 1314, 1351); T6_total and T7_2h_total return 0 for the
  // infinite survey before reaching those checks (:849-850, :1048-1049)
  if (calc[2] && geom != TP_GEOM_INFINITE) cli::die("T4: Wrong survey geometry, only coded for infinite survey", -1);
  if (calc[3] && geom != TP_GEOM_INFINITE) cli::die("T5: Wrong survey geometry, only coded for infinite survey", -1);
  if (calc[4] && geom == TP_GEOM_CIRCLE)
    cli::die("T6: Wrong survey geometry, only coded for square and rectangular survey", -1);
  if (calc[5] && geom != TP_GEOM_INFINITE) cli::die("T7: Wrong survey geometry, only coded for infinite survey", -1);
  if (calc[6] && (geom == TP_GEOM_CIRCLE || geom == TP_GEOM_RECTANGLE))
    cli::die("T7_SSC: Wrong survey geometry, only coded for square survey", -1);

  tp_ctx* ctx = cli::make_context(cosmo_file, nz_file, 0, nullptr);
  cli::check(tp_set_shape_noise(ctx, par.shapenoise_sigma, par.galaxy_density, par.shapenoise_only),
             "shape noise", ctx);
  if (geom == TP_GEOM_RECTANGLE) cli::check(tp_set_rectangle_side(ctx, par.theta_max_smaller), "thetaMax_smaller", ctx);

  std::vector<double> thetas(4096);
  int n = 0;
  cli::check(tp_read_thetas(thetas_file.c_str(), thetas.data(), (int)thetas.size(), &n), "reading " + thetas_file);
  if (n > (int)thetas.size()) cli::die("too many aperture radii in " + thetas_file, -1);

  std::vector<double> combis;  // independent triplets theta1 <= theta2 <= theta3 (:155-170)
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++)
      for (int k = j; k < n; k++)
        for (int t : {i, j, k}) {
          double r;
          cli::check(tp_convert_angle_to_rad(thetas[t], "arcmin", &r), "converting radii");
          combis.push_back(r);
        }
  const int n_ind = (int)(combis.size() / 3);
  std::vector<double> a, b;  // pairs (i, j >= i) in the reference's order
  for (int i = 0; i < n_ind; i++)
    for (int j = i; j < n_ind; j++) {
      a.insert(a.end(), combis.begin() + 3 * i, combis.begin() + 3 * i + 3);
      b.insert(b.end(), combis.begin() + 3 * j, combis.begin() + 3 * j + 3);
    }
  const int npair = (int)(a.size() / 3);

  char filename[255];
  const double n_deg = par.galaxy_density / cli::rad_to_deg(1) / cli::rad_to_deg(1);
  const double theta_max_deg = cli::rad_to_deg(par.theta_max);
  const int terms[7] = {1, 2, 4, 5, 6, 7, 72};
  for (int q = 0; q < 7; ++q) {
    if (!calc[q]) continue;
    std::vector<double> cov(npair, 0.0);
    if (terms[q] == 72) {
      // T7_2h: zero (see the header comment)
      snprintf(filename, sizeof(filename), "cov_%s_term7_2h_Numerical_sigma_%.2f_n_%.2f_thetaMax_%.2f_gpu.dat",
               type_str.c_str(), par.shapenoise_sigma, n_deg, theta_max_deg);
    } else {
      int ncap = 0;
      int st = tp_cov_total_batch(ctx, 0, terms[q], geom, par.theta_max, par.area, a.data(), b.data(), npair,
                                  precision, cov.data(), &ncap);
      if (st == TP_ERR_CAPACITY)
        std::cerr << "warning: " << tp_last_error(ctx) << std::endl;
      else
        cli::check(st, std::string("T") + std::to_string(terms[q]), ctx);
      snprintf(filename, sizeof(filename), "cov_%s_term%dNumerical_sigma_%.2f_n_%.2f_thetaMax_%.2f_gpu.dat",
               type_str.c_str(), terms[q], par.shapenoise_sigma, n_deg, theta_max_deg);
    }
    std::cerr << "Writing " << names[q] << " to " << out_folder + filename << std::endl;
    if (!write_cov(cov, n_ind, out_folder + filename)) {
      std::cerr << "writeCov: Could not open " << out_folder + filename << std::endl;
      std::cerr << "Writing instead to current directory!" << std::endl;
      if (!write_cov(cov, n_ind, filename)) cli::die(std::string("writeCov: Could not open ") + filename, -1);
    }
  }
  tp_ctx_destroy(ctx);
  return 0;
}
