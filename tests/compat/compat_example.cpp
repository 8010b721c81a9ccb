// A caller of the reference's C++ API, compiled against
// include/threepoint_gb300_compat.hpp: the calls and globals of
// calculateApertureStatistics.cu, calculateGamma.cu and
// calculateApertureStatisticsCovariance.cu, one value each.
//   compat_example cosmo.param nz.dat [halo]
// prints: Map3(8',8',16')  Re Gamma0  Im Gamma0  T2_total(square)
// [and, with "halo", T7_total(infinite) after initHalomodel, as the
// covariance driver calls them]
#include <cstdio>
#include <string>

#include "threepoint_gb300_compat.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    cosmology cosmo(argv[1]);
    std::vector<double> nz;
    read_n_of_z(argv[2], 256, cosmo.zmax, nz);
    copyConstants();
    set_cosmology(cosmo, &nz);
    const double a = convert_angle_to_rad(8), b = convert_angle_to_rad(16);
    double m3 = MapMapMap({a, a, b});
    compute_weights_bessel();
    std::complex<double> g0 = gamma0(a, a, 0.5 * a, z_max);
    type = 1;
    thetaMax = convert_angle_to_rad(10, "deg");
    area = thetaMax * thetaMax;
    sigma = 0.3;
    n = 10 / convert_angle_to_rad(1) / convert_angle_to_rad(1);
    constant_powerspectrum = true;
    lMin = 0;
    initCovariance();
    double t2 = T2_total({a, a, b}, {a, b, b});
    printf("%.17g %.17g %.17g %.17g\n", m3, g0.real(), g0.imag(), t2);
    if (argc > 3 && std::string(argv[3]) == "halo") {
      constant_powerspectrum = false;
      type = 2;
      initCovariance();
      initHalomodel();
      printf("%.17g %.17g\n", T7_total({a, a, b}, {a, b, b}), T7_2h_total({a, a, b}, {a, b, b}));
    }
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
