// Device harness around the reference's OWN device code, used only to pin the
// oracle and the GPU path (test infrastructure; built by `make -C oracle
// refdev REF=<reference cuda_version directory>` into oracle/_ref/ as a
// device-only cubin, never shipped, never linked into the product).
//
// It compiles the reference's cuda_version/bispectrum.cu, gamma.cu and
// halomodel.cu as they are (the GSL host routines of gamma.cu are declared by
// oracle/gsl_stub and never called) and adds kernels that call the
// reference's __device__ functions at caller-given points:
//   ref_node_eval    bispec(ell/f_K(z), z, idx, didx) (bispectrum.cu:221-291) and
//                    integrand_bkappa(z, ell) (:311-333), idx/didx/f_K formed as
//                    integrand_bkappa forms them (:320-324)
//   ref_gamma_points the sum over the Ogata nodes k = 1..prec_k-1 of
//                    full_integrand_gamma0/1 (gamma.cu:419-482) at (z, phi, psi),
//                    reduced in the pairwise order of compute_integrand_gamma0/1's
//                    shared-memory reduction (:267-363)
//   ref_halo_los     the one-halo line-of-sight tri- and pentaspectrum
//                    (halomodel.cu:430-510) with the mass tables the
//                    reference's host code built
// The host uploads the constants that copyConstants / set_cosmology /
// compute_weights_bessel would upload (bispectrum.cu:90-219, gamma.cu:13-56),
// from tables the reference's own host code built (oracle/ref_harness.cu).
//
// Every z the caller passes must lie in [dz/2, z_max): below half a bin the
// reference's mid-bin interpolation reads table index -1
// (bispectrum.cu:356-359, 389-392, 421-424), and z = z_max reads index 256.
#include "bispectrum.cu"
#include "gamma.cu"
#include "halomodel.cu"

// halomodel.cu's device code reads this survey-variance table, which
// apertureStatisticsCovariance.cu defines; that file is not compiled here.
__constant__ double dev_sigma2_from_windowfunction_array[n_redshift_bins];

// trispectrum_limber_integrated(0, z_max, m, l1..l4) and
// pentaspectrum_limber_integrated(0, z_max, m, l1..l6) (halomodel.cu:430-510)
// at rows pts[n][7] = (m, l1, ..., l6)
extern "C" __global__ void ref_halo_los(const double* pts, int n, double* tri, double* penta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = pts + 7 * i;
  tri[i] = trispectrum_limber_integrated(0, dev_z_max, p[0], p[1], p[2], p[3], p[4]);
  penta[i] = pentaspectrum_limber_integrated(0, dev_z_max, p[0], p[1], p[2], p[3], p[4], p[5], p[6]);
}

extern "C" __global__ void ref_node_eval(const double* ell, const double* z, int n_tri, int n_z, double* bis,
                                         double* integ) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n_tri * n_z) return;
  const int i = (int)(t / n_z), j = (int)(t % n_z);
  const double zz = z[j], l1 = ell[3 * i], l2 = ell[3 * i + 1], l3 = ell[3 * i + 2];
  double didx = zz / dev_z_max * (dev_n_redshift_bins);
  int idx = didx;
  didx = didx - idx;
  const double fk = f_K_interpolated(idx, didx);
  bis[t] = bispec(l1 / fk, l2 / fk, l3 / fk, zz, idx, didx);
  integ[t] = integrand_bkappa(zz, l1, l2, l3);
}

extern "C" __global__ void ref_gamma_points(const double* pts, int n, double x1, double x2, double x3, int which,
                                            double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double z = pts[3 * i], phi = pts[3 * i + 1], psi = pts[3 * i + 2];
  cuDoubleComplex v[prec_k - 1];
  for (int k = 1; k < prec_k; ++k)
    v[k - 1] = which == 0 ? full_integrand_gamma0(phi, psi, z, k, x1, x2, x3)
                          : full_integrand_gamma1(phi, psi, z, k, x1, x2, x3);
  for (int size = (prec_k - 1) / 2; size > 0; size /= 2)
    for (int j = 0; j < size; ++j) v[j] = cuCadd(v[j], v[j + size]);
  out[2 * i] = cuCreal(v[0]);
  out[2 * i + 1] = cuCimag(v[0]);
}
