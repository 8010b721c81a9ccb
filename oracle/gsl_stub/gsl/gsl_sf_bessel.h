/* Declarations only, for compiling the reference's gamma.cu device code in
 * oracle/ref_device.cu where GSL is not installed. The device functions the
 * harness calls never reach these host routines, and the harness is built
 * as a device-only object (-cubin), so nothing is linked against them. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_zero_Jnu(double nu, unsigned int s);
double gsl_sf_bessel_Jn(const int n, const double x);
double gsl_sf_bessel_J1(const double x);
#ifdef __cplusplus
}
#endif
