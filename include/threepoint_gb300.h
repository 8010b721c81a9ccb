/*
 * threepoint_gb300 -- C ABI of the GB300 (sm_103a) implementation of the
 * threepoint model-evaluation path: the line-of-sight projected BiHalofit
 * convergence bispectrum b_kappa, <Map^3>, the shear-3PCF natural components
 * Gamma_i and the <Map^3> covariance terms T1, T2, T4.
 *
 * Conventions: plain pointers and sizes; host buffers unless a name ends in
 * _device; angles in radians; FP64 results. Every call returns an int status
 * (TP_OK == 0) and never exits the process; tp_status_string() and
 * tp_last_error() describe failures. One context = one CUDA device + one
 * stream; calls on one context are not thread-safe.
 *
 * Each entry point names the reference interface it replaces (file:line in
 * the reference project sheydenreich/threepoint).
 */
#ifndef THREEPOINT_GB300_H
#define THREEPOINT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  TP_OK = 0,
  TP_ERR_ARG = 1,         /* invalid argument */
  TP_ERR_IO = 2,          /* file missing or unreadable */
  TP_ERR_FORMAT = 3,      /* file content not in the expected format */
  TP_ERR_CUDA = 4,        /* CUDA runtime error */
  TP_ERR_STATE = 5,       /* call out of order (e.g. no cosmology set) */
  TP_ERR_CAPACITY = 6,    /* an adaptive integral hit its region/sweep cap */
  TP_ERR_NOMEM = 7
};

/* precision of the integrand evaluation */
enum {
  TP_FP64 = 0,  /* plain FP64 BiHalofit: the correctness path */
  TP_FP32 = 1   /* FP32 BiHalofit with compensated (Kahan) line-of-sight sums */
};

/* error norm of a vector integrand (cubature.h) */
enum { TP_NORM_INDIVIDUAL = 0, TP_NORM_PAIRED, TP_NORM_L2, TP_NORM_L1, TP_NORM_LINF };

/* survey geometry of the covariance (calculateApertureStatisticsCovariance.cu:111-130);
 * the rectangle's second side is set by tp_set_rectangle_side */
enum { TP_GEOM_CIRCLE = 0, TP_GEOM_SQUARE = 1, TP_GEOM_INFINITE = 2, TP_GEOM_RECTANGLE = 3 };

/* Cosmological parameters; same fields and meaning as the reference's class
 * cosmology (cuda_version/cosmology.cuh:13-29). */
typedef struct {
  double h, sigma8, omb, omc, ns, w, om, ow, zmax;
} tp_cosmology;

typedef struct tp_ctx tp_ctx;

const char* tp_status_string(int status);
const char* tp_last_error(const tp_ctx* ctx);
/* library version string */
const char* tp_version(void);

/* ---- inputs (host only, no GPU needed) --------------------------------- */

/* Replaces cosmology::cosmology(const std::string&) (cuda_version/cosmology.cu:11-78):
 * reads h, sigma_8, Omega_b, n_s, w, Omega_m, z_max; sets ow = 1-om, omc = om-omb. */
int tp_cosmology_from_file(const char* path, tp_cosmology* out);

/* Replaces read_n_of_z (cuda_version/helpers.cu:9-128): rebins an ASCII
 * "z n(z)" table to n_bins bins at i*zmax/n_bins and normalises sum(n)*dz=1. */
int tp_read_n_of_z(const char* path, int n_bins, double zmax, double* nz_out);

/* The rebinning/normalisation step of read_n_of_z applied to an in-memory
 * table of nf (z, n) pairs with uniform z spacing. */
int tp_rebin_n_of_z(const double* z, const double* n, int nf, int n_bins, double zmax, double* nz_out);

/* Replaces read_thetas (cuda_version/helpers.cu:176-200): one value per line.
 * Writes at most cap values, *n_out = number read. */
int tp_read_thetas(const char* path, double* out, int cap, int* n_out);

/* convert_angle_to_rad (cuda_version/helpers.cu:130-153); unit "arcmin", "deg" or "rad" */
int tp_convert_angle_to_rad(double value, const char* unit, double* out);

/* Survey parameters of the covariance; same fields as the reference's class
 * covarianceParameters (cuda_version/cosmology.cuh:44-56), angles in rad,
 * density in rad^-2, area in rad^2. */
typedef struct {
  double theta_max, theta_max_smaller, shapenoise_sigma, galaxy_density, area;
  int shapenoise_only;
} tp_cov_params;

/* Replaces covarianceParameters::covarianceParameters(fn) (cuda_version/cosmology.cu:92-170):
 * "name value" lines (thetaMax, thetaMax_smaller, shapenoise_sigma,
 * galaxy_density, unit, shapenoiseOnly, area), '#' comments; converts to rad
 * with the file's unit. Unlike the reference, an unknown name or unit is an
 * error (TP_ERR_FORMAT) instead of a message and half-converted values. */
int tp_cov_params_from_file(const char* path, tp_cov_params* out);

/* (r, u, v) binning of the shear 3PCF; the reference's struct configGamma
 * (cuda_version/helpers.cuh:48-52), r in arcmin. */
typedef struct {
  int rsteps, usteps, vsteps;
  double umin, umax, vmin, vmax, rmin, rmax;
} tp_gamma_config;

/* Replaces read_gamma_config (cuda_version/helpers.cu:242-318): "name value"
 * lines rmin, rmax, umin, umax, vmin, vmax, rsteps, usteps, vsteps. An unknown
 * name is TP_ERR_FORMAT (the reference prints a message and stops reading). */
int tp_gamma_config_from_file(const char* path, tp_gamma_config* out);

/* Triangles of the bin centres of calculateGamma (cuda_version/calculateGamma.cu:104-121),
 * r-major, then u, then v: r log-spaced, u and v linear; r2 = r [arcmin -> rad],
 * r3 = u r2, r1 = v r3 + r2. x_out[3i..3i+2] = (r1, r2, r3) [rad],
 * ruv_out[3i..3i+2] = (r [arcmin], u, v); ruv_out may be NULL. */
int tp_gamma_triangles(const tp_gamma_config* cfg, double* x_out, double* ruv_out);

/* ---- context ------------------------------------------------------------ */
int tp_ctx_create(int device, tp_ctx** out);
int tp_ctx_destroy(tp_ctx* ctx);
/* the context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or CUDA events with the library's asynchronous entry points */
void* tp_ctx_stream(tp_ctx* ctx);

/* Limits of the adaptive integrals run on this context: region_cap = regions
 * per integral (default 32768; an integral that needs more stops there, see
 * tp_ctx_set_escalation), max_ctas = CTAs of the persistent grid (0 = all resident).
 * Device scratch = grid * region_cap * ~90 bytes (3-D integrands). */
int tp_ctx_set_limits(tp_ctx* ctx, int region_cap, int max_ctas);

/* The reference's cubature has no region cap (hcubature_v with maxEval = 0,
 * apertureStatistics.cu:222-225, gamma.cu:110). The host-API calls
 * tp_map3_batch and tp_gamma_batch therefore integrate the integrals that
 * reach region_cap again, from the start, with 16x the cap (fewer CTAs, the
 * region stores bounded to 32 GB), until they converge or reach
 * max_region_cap (default 2^24); since the adaptive sequence is
 * deterministic, the result is the one an uncapped run gives. Only integrals
 * that still reach max_region_cap are reported (status bit 1,
 * TP_ERR_CAPACITY). max_region_cap <= region_cap turns this off. */
int tp_ctx_set_escalation(tp_ctx* ctx, int max_region_cap);

/* Measured throughput of the pipes that bound the integrand kernels, whole
 * device: out[0] ex2.approx.f32 (SFU) ops/s, out[1] FP32 FMA/s, out[2] FP64 FMA/s. */
int tp_pipe_peaks(int device, double* out);

/* Replaces copyConstants() + set_cosmology(cosmo, nz, Pk, dk, kmin, kmax)
 * (cuda_version/bispectrum.cu:90-219), batched: builds on the GPU, in FP64,
 * the z-tables (f_K, g, D1, r_sigma, n_eff, ncur) of n_cosmo cosmologies and
 * the per-node line-of-sight coefficients derived from them.
 *   nz: 256 values per cosmology (nz_stride = 256) or one shared row
 *       (nz_stride = 0), as produced by tp_read_n_of_z.
 *   pk: optional (NULL -> Eisenstein & Hu): 256 log-spaced linear P(k) values
 *       per cosmology with dk, kmin, kmax as from convert_Pk (helpers.cu:202-214).
 *       As in the reference, the table is read only by the bispectrum's and
 *       P(ell)'s linear P(k) (bispectrum.cu:605-621); the sigma_8
 *       normalisation and the non-linear scales r_sigma, n_eff, ncur still
 *       come from Eisenstein & Hu, because the reference's set_cosmology
 *       declares a local Pk_given (:132) that hides the global flag its host
 *       code reads (:36, :623). */
int tp_set_cosmologies(tp_ctx* ctx, const tp_cosmology* cosmo, int n_cosmo, const double* nz, int nz_stride,
                       const double* pk, double dk, double kmin, double kmax);

/* Shape noise and galaxy density used by the power spectrum P(ell) of the
 * covariance (globals sigma, n, constant_powerspectrum of the reference:
 * bispectrum.cu:21-23, initCovariance apertureStatisticsCovariance.cu:30-45). */
int tp_set_shape_noise(tp_ctx* ctx, double sigma_eps, double n_gal_per_rad2, int constant_powerspectrum);

/* Smaller side [rad] of a rectangular survey (TP_GEOM_RECTANGLE), the global
 * thetaMax_smaller of the reference (apertureStatisticsCovariance.cu:24,154-172):
 * the window is sinc^2(lx*theta_max/2) * sinc^2(ly*theta_max_smaller/2). */
int tp_set_rectangle_side(tp_ctx* ctx, double theta_max_smaller);

/* Copies cosmology i's FP64 tables to the host: 6*256 doubles
 * (f_K, g, D1, r_sigma, n_eff, ncur) followed by norm. */
int tp_get_tables(tp_ctx* ctx, int cosmo_index, double* out);

/* ---- point evaluations (no cubature) ------------------------------------ */

/* bkappa(ell1, ell2, ell3) (cuda_version/bispectrum.cu:293-309) for n points:
 * ell is [n][3], cosmo_index[n] selects the cosmology (NULL -> cosmology 0). */
int tp_bkappa_batch(tp_ctx* ctx, const int* cosmo_index, const double* ell, long n, int precision, double* out);

/* Pell(ell) (cuda_version/bispectrum.cu:511-529, device branch) for n values. */
int tp_pell_batch(tp_ctx* ctx, int cosmo_index, const double* ell, long n, int precision, double* out);

/* The 96 line-of-sight terms of bkappa (GQ96_of_bdelta, cuda_version/bispectrum.cu:293-309)
 * for n triangles ell[n][3] of one cosmology, evaluated by the functions the
 * integration kernels use: term[i*96 + j] = W96 * z_max/2 * 27/8 Om^3 (H0/c)^5 *
 * integrand_bkappa(z_j, ell) (:311-333) at Gauss node j (j even: z_max/2 (1 - a_{j/2}),
 * odd: z_max/2 (1 + a_{j/2})), so a triangle's terms sum to bkappa; bispec
 * (optional, same shape) receives bispec(ell/f_K(z_j), z_j) (:221-291). */
int tp_bkappa_nodes(tp_ctx* ctx, int cosmo_index, const double* ell, long n, int precision, double* term,
                    double* bispec);

/* The Gamma cubature integrand at n points pts[n][3] = (z, phi, psi) of the
 * triangle x[3] (radians): out[2i], out[2i+1] = real and imaginary part of the
 * sum over the Ogata nodes k = 1..32 of full_integrand_gamma0 (which = 0) or
 * full_integrand_gamma1 (which = 1) (cuda_version/gamma.cu:267-363, 419-482),
 * before the cubature and the outer prefactor. */
int tp_gamma_integrand_points(tp_ctx* ctx, int cosmo_index, const double* x, int which, const double* pts, int n,
                              int precision, double* out);

/* ---- adaptive integrals ------------------------------------------------- */

/* Replaces MapMapMap(thetas, phiMin, phiMax, lMin) (cuda_version/apertureStatistics.cu:201-230;
 * declared apertureStatistics.cuh:106) for every (cosmology, triplet) pair:
 * out[c * n_trip + t] = <Map^3>(thetas[3t..3t+2]) of cosmology c, by
 * h-adaptive Genz-Malik cubature over (l1, l2, phi) on [lMin, lMax]^2 x
 * [phiMin, phiMax] with relative tolerance rel_tol (reference: 1e-4),
 * divided by (2 pi)^3. lMax <= 0 selects the reference bound 10/theta_min.
 * err (optional) receives the error estimate, neval (optional) the number of
 * integrand points. Returns TP_ERR_CAPACITY if any integral hit a cap (its
 * value is still written; status_out[i] != 0 flags which, if given). */
int tp_map3_batch(tp_ctx* ctx, const int* cosmo_index, int n_cosmo, const double* thetas, int n_trip,
                  double phi_min, double phi_max, double l_min, double l_max, double rel_tol, int precision,
                  double* out, double* err, int64_t* neval, int* status_out);

/* Same as tp_map3_batch with device-resident inputs/outputs, asynchronous on
 * the context stream (no host synchronisation). job_cosmo/job_theta are
 * [n_jobs] and [n_jobs][3] device arrays; out/err are [n_jobs]; neval, nlive
 * and status are [n_jobs] (each may be NULL). nlive counts the cubature points
 * whose filter product is non-zero, i.e. whose line-of-sight sum was evaluated.
 * job_order (optional, [n_jobs] device permutation) is the order in which the
 * persistent grid takes the jobs: putting the most expensive integrals first
 * shortens the tail of the launch (tp_map3_batch does this itself from the
 * costs it has seen). Results are always written at the job's own index. */
int tp_map3_jobs_device(tp_ctx* ctx, const int* job_cosmo_device, const double* job_theta_device, int n_jobs,
                        double phi_min, double phi_max, double l_min, double l_max, double rel_tol, int precision,
                        double* out_device, double* err_device, int64_t* neval_device, int64_t* nlive_device,
                        int* status_device, const int* job_order_device);

/* Allocation-free variant of tp_map3_jobs_device; no counterpart in the
 * reference. For callers that cannot allocate device memory when they
 * integrate (inside CUDA stream capture, under a framework-owned allocator,
 * in pipelines that forbid allocation after start-up): it calls no cudaMalloc
 * or cudaFree and keeps the per-CTA region stores in a fixed 128 MiB
 * __device__ array of the library (held on every GPU that loads the library
 * until exit). Limits: at most 8192 regions per integral and a grid trimmed
 * to fit the array (192 CTAs). An integral that needs more regions stops at
 * the cap with bit 1 set in its status_device entry (bit 2: not converged
 * within the sweep limit) and its value still written; the call itself
 * returns TP_OK then, not TP_ERR_CAPACITY. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress): make it
 * before any stream capture. All calls share the array, so calls that overlap
 * on the GPU race; serialise them. Inputs, outputs and the context's
 * cosmology tables are the caller's/the context's, as in tp_map3_jobs_device. */
int tp_map3_jobs_noalloc(tp_ctx* ctx, const int* job_cosmo_device, const double* job_theta_device, int n_jobs,
                         double phi_min, double phi_max, double l_min, double l_max, double rel_tol, int precision,
                         double* out_device, double* err_device, int* status_device);

/* Replaces gamma0..gamma3(x1, x2, x3, z_max) (cuda_version/gamma.cu:98-148;
 * gamma.cuh:56-97): natural components of the shear 3PCF for n triangles
 * x[3i..3i+2] (radians) of one cosmology, by Ogata Hankel quadrature
 * (h = 0.1, 32 nodes) inside a 3-D adaptive cubature over (z, phi, psi) with
 * relative tolerance rel_tol (reference: 1e-3). comp_mask bit k selects
 * Gamma^k; out is [n][4] complex as 8 doubles (re, im per component); the
 * orthocentre-to-centroid rotation is applied (gamma.cuh:25). */
int tp_gamma_batch(tp_ctx* ctx, int cosmo_index, const double* x, int n, int comp_mask, double rel_tol,
                   int precision, double* out, int* status_out);

/* ---- FFT aperture-mass measurement ------------------------------------- */

/* Replaces the reference's Python measurement side (python_scripts/
 * aperture_mass_computer.py): class aperture_mass_computer(npix, theta_ap,
 * fieldsize, use_polynomial_filter) (:19-372) and extract_Map3 /
 * extract_Map3_of_field (:375-531). One tp_apm holds a grid of npix x npix
 * pixels over a square field of side fieldsize, the n_theta aperture radii
 * (fieldsize and thetas in the same unit, arcmin in the reference) and the
 * filter (polynomial != 0: Schneider's polynomial filter, else the
 * exponential one); it keeps on the device the Fourier transforms of the filter
 * grids of every aperture, so only the field's own transforms are done per
 * field. precision TP_FP64 does the transforms and Fourier products in FP64
 * (the reference's numpy precision); TP_FP32 does them in FP32 (gridding, maps
 * and the <Map^3> sums stay FP64). Needs cuFFT at run time (loaded with
 * dlopen; TP_ERR_STATE if absent). */
typedef struct tp_apm tp_apm;
int tp_apm_create(tp_ctx* ctx, int npix, double fieldsize, const double* thetas, int n_theta, int polynomial,
                  int precision, tp_apm** out);
/* A tp_apm's calls need its context; destroying it does not (it may come
 * after tp_ctx_destroy). */
int tp_apm_destroy(tp_apm* apm);
/* FFT grid side F >= 2 npix - 1 of the zero-padded convolutions */
int tp_apm_fft_size(const tp_apm* apm);

/* normalize_shear(Xs, Ys, shears, CIC=True, normalize=False) (:288-372):
 * cloud-in-cell gridding of n_gal galaxies at (x, y) with shears g1 + i g2 on
 * numpy.histogram2d's bins (edges i/(npix-1)*fieldsize); the shear-sum and
 * weight grids stay in the tp_apm (row-major [x bin][y bin]). Host arrays; the
 * _device form takes device arrays and does not synchronise. */
int tp_apm_grid(tp_apm* apm, const double* x, const double* y, const double* g1, const double* g2, long n_gal);
int tp_apm_grid_device(tp_apm* apm, const double* x_device, const double* y_device, const double* g1_device,
                       const double* g2_device, long n_gal);
/* set / read the gridded shear sums (re, im) and weights, npix*npix each */
int tp_apm_set_grid(tp_apm* apm, const double* shear_re, const double* shear_im, const double* weight);
int tp_apm_get_grid(tp_apm* apm, double* shear_re, double* shear_im, double* weight);

/* Map_fft(gamma, norm=weights, normalize_weighted=True, periodic_boundary=False)
 * (:199-286) for every aperture: maps[t][npix][npix] = (Im g * Im Q - Re g * Re Q)
 * / (w * |Q|), '*' the zero-padded FFT convolution cropped to the grid
 * (scipy.signal.fftconvolve 'same'); mcross (optional, return_mcross) =
 * -(Re g * Im Q + Im g * Re Q) / (w * |Q|). Either output may be NULL. */
int tp_apm_maps(tp_apm* apm, double* maps, double* mcross);

/* Map_fft_from_kappa(kappa) (:183-197) for every aperture: maps[t] =
 * fftconvolve(kappa, U_t, 'same') * fieldsize^2 / npix^2 with the exponential
 * U filter (Ufunc, :72-80); kappa is npix*npix host values. The maps become
 * the ones tp_apm_map3 reads. */
int tp_apm_maps_from_kappa(tp_apm* apm, const double* kappa, double* maps);

/* The <Map^3> part of extract_Map3_of_field (:466-531) over the maps of the
 * last tp_apm_maps / extract call: out[q] for every triplet i <= j <= k of the
 * apertures (in the order of the reference's loops) = the mean of
 * M_i M_j M_k over [c, npix - c)^2, c = round(theta / fieldsize * npix * f)
 * with f = 4 (exponential) or 1 (polynomial) and theta = theta_k, or the
 * largest aperture when same_fieldsize != 0. */
int tp_apm_map3(tp_apm* apm, int same_fieldsize, double* out);

/* extract_Map3(Xs, Ys, shear_catalogue, npix, thetas, fieldsize) (:375-405):
 * gridding, maps and <Map^3> in one call, host catalogue in, host results out;
 * the _device form reads device arrays and writes out_device asynchronously. */
int tp_apm_extract_map3(tp_apm* apm, const double* x, const double* y, const double* g1, const double* g2, long n_gal,
                        int same_fieldsize, double* out);
int tp_apm_extract_map3_device(tp_apm* apm, const double* x_device, const double* y_device, const double* g1_device,
                               const double* g2_device, long n_gal, int same_fieldsize, double* out_device);

/* Ogata nodes/weights of compute_weights_bessel (cuda_version/gamma.cu:13-56):
 * out[4][33] = psi(J6), product(J6), psi(J2), product(J2). */
int tp_ogata_weights(double* out);

/* Covariance terms of <Map^3> (cuda_version/apertureStatisticsCovariance.cu):
 * T1_total, T2_total, T4_total (:272-683) and the halo-model terms
 * T5_total, T6_total, T7_total (:685-1044) for pairs of triplets.
 * term: 1, 2, 4, 5, 6 or 7; geometry TP_GEOM_*; theta_max [rad] and area
 * [rad^2] as in covarianceParameters (cosmology.cu:92-170).
 * out[i] = T_term(th123[i], th456[i]). T5 and T7 exist for the infinite
 * geometry only, T6 for the square and the rectangle (0 for the infinite
 * geometry, as T6_total returns); the others are TP_ERR_ARG, where the
 * reference throws. precision TP_FP64 is the reference's arithmetic; with
 * TP_FP32 the line-of-sight node sums run in FP32 (the cubature stays FP64). */
int tp_cov_total_batch(tp_ctx* ctx, int cosmo_index, int term, int geometry, double theta_max, double area,
                       const double* th123, const double* th456, int n, int precision, double* out,
                       int* n_capped);

/* Single covariance terms T1, T2, T4, T5, T6, T7 of (th1..th6)
 * (apertureStatisticsCovariance.cu:1065-1313) for n six-tuples th6[n][6],
 * without the permutation sums. T2 is 0 for the infinite geometry; T4 exists
 * only for the infinite geometry (normalised by area), as in the reference,
 * whose T4 throws for the others (TP_ERR_ARG here). *n_capped (optional)
 * receives the number of integrals that hit a cap. */
int tp_cov_term_batch(tp_ctx* ctx, int cosmo_index, int term, int geometry, double theta_max, double area,
                      const double* th6, int n, int precision, double* out, int* n_capped);

/* The argument patterns of T_term_total(th123, th456) as this library sums
 * them (the reference's T1/T2/T4/T5/T6/T7_total branches): for k < return
 * value, multiplicity mult[k] times T_term of the radii (a0, a1, a2, b0, b1,
 * b2)[idx[6k + j]], j < 6. Host only; -1 for a bad term or fewer than needed
 * entries (cap); 0 terms for T2 and T6 of the infinite geometry. */
int tp_cov_total_terms(int term, int geometry, const double* th123, const double* th456, int* mult, int* idx,
                       int cap);

/* Relative tolerance of the T5 / T6 / T7 integrals (term 5..7); 0 restores
 * the reference's 1e-2 / 1e-1 / 1e-1 (apertureStatisticsCovariance.cu:1222,
 * 1271, 1307). */
int tp_ctx_set_cov_tolerance(tp_ctx* ctx, int term, double rel_tol);

/* CTAs that integrate one T5/T6/T7 integral together: 16 (default: a
 * thread-block cluster of 16 CTAs, a non-portable cluster size, when the batch
 * has at most 1/16 as many integrals as the device has CTA slots, else 8), 8
 * (8-CTA clusters) or 1 (one CTA per integral). A cluster deals out each
 * sweep's regions to its CTAs; the results are the same bit for bit. */
int tp_ctx_set_halo_cluster(tp_ctx* ctx, int ctas);

/* <Map^3> calls (tp_map3_batch, tp_map3_jobs_device) with no more integrals
 * than the device has CTA slots run one 8-CTA cluster per integral when on
 * (1, default); 2 uses clusters for every batch, 0 one CTA per integral
 * always. Same results bit for bit. */
int tp_ctx_set_map3_cluster(tp_ctx* ctx, int on);

/* Halo model of T5-T7 (cuda_version/halomodel.cu), built per cosmology on
 * first use.
 * tp_halo_tables: out[0..127] = sigma^2(m_i), out[128..255] = dsigma^2/dm(m_i)
 *   at z = 0, m_i = 10^(9 + i/16) Msun/h (setSigma2 / setdSigma2dm, :197-276).
 * tp_halo_los: at rows pts[n][7] = (m, l1, ..., l6), m in [1e9, 1e17]:
 *   tri[i] = trispectrum_limber_integrated(0, z_max, m, l1..l4) and
 *   penta[i] = pentaspectrum_limber_integrated(0, z_max, m, l1..l6) (:430-510).
 * tp_halo_integrand_points: the integrand of T5 (x rows of 6: ln l1, ln l2,
 *   ln l5, phi1, phi2, m), T6 (rows of 7: ln l3, ln l4, ln l5, phi3, phi4,
 *   phi5, m; geometry square or rectangle) or T7 (rows of 7: ln l1, ln l2,
 *   ln l4, ln l5, phi1, phi2, m) for the radii th6 (integrand_T5_infinite,
 *   integrand_T6_square / _rectangle, integrand_T7_infinite, :2151-2314),
 *   before the 1/area/(2 pi)^n factors. */
int tp_halo_tables(tp_ctx* ctx, int cosmo_index, double* out);
int tp_halo_los(tp_ctx* ctx, int cosmo_index, const double* pts, long n, int precision, double* tri, double* penta);
int tp_halo_integrand_points(tp_ctx* ctx, int cosmo_index, int term, int geometry, double theta_max,
                             const double* th6, const double* x, long n, int precision, double* out);

/* ---- likelihood of <Map^3> model vectors -------------------------------- */

/* Gaussian likelihood of the reference's cosmosis likelihood module
 * (cosmosis/threepoint_likelihood.py:8-58): chi2 = (m - d)^T C^-1 (m - d),
 * log L = -chi2 / 2. tp_likelihood_create factors the n x n covariance (FP64
 * Cholesky on the GPU) once; TP_ERR_ARG if it is not positive definite (the
 * reference inverts any invertible matrix with numpy). */
typedef struct tp_likelihood tp_likelihood;
int tp_likelihood_create(int device, const double* data, const double* cov, int n, tp_likelihood** out);
void tp_likelihood_destroy(tp_likelihood* lk);
const char* tp_likelihood_last_error(const tp_likelihood* lk);
/* C^-1 (n x n, row-major), the file the reference writes as cov_inv */
int tp_likelihood_cov_inv(tp_likelihood* lk, double* out);
/* chi2 of n_models model vectors models[n_models][n] (host buffers) */
int tp_likelihood_chi2(tp_likelihood* lk, const double* models, int n_models, double* chi2_out);
/* Device-resident form, asynchronous on `stream` (a cudaStream_t; NULL = the
 * likelihood's own stream): model b at models_device + b * ld, ld >= n. */
int tp_likelihood_chi2_device(tp_likelihood* lk, const double* models_device, int n_models, long ld,
                              double* chi2_device, void* stream);

/* ---- surrogate network of log b_kappa ----------------------------------- */

/* A multilayer perceptron 8 -> 256 -> 256 -> 256 -> 256 -> 1 (SiLU after the
 * hidden layers, linear output) on the tensor cores: BF16 operands, FP32
 * accumulation, FP32 master parameters and Adam moments. It has no
 * counterpart in the reference; its inputs are the 8 scaled features of a
 * (triangle, cosmology) point and its output the scaled log b_kappa
 * (threepoint_gb300/surrogate.py defines the scaling). Parameters travel as
 * one flat FP64 array: W1 [256][8], b1 [256], W2, W3, W4 [256][256] with their
 * biases, W5 [1][256], b5 [1] (tp_mlp_param_count() values; W[out][in]).
 * Loss: mean squared error. Every call runs on the network's own stream;
 * max_batch bounds one forward / gradient / training batch. */
typedef struct tp_mlp tp_mlp;
long tp_mlp_param_count(void);
/* on failure *out is NULL (TP_ERR_ARG: max_batch outside [1, 2^22]) */
int tp_mlp_create(int device, int max_batch, tp_mlp** out);
void tp_mlp_destroy(tp_mlp* m);
const char* tp_mlp_last_error(const tp_mlp* m);
int tp_mlp_set_params(tp_mlp* m, const double* params);
int tp_mlp_get_params(tp_mlp* m, double* params);
/* y[n] for features x[n][8] (host buffers; any n, in batches of max_batch) */
int tp_mlp_forward(tp_mlp* m, const double* x, long n, double* y);
/* loss and its gradient (flat, the parameter layout) on one batch, no update */
int tp_mlp_gradients(tp_mlp* m, const double* x, const double* t, long n, double* grads, double* loss);
/* one Adam step (Kingma & Ba 2015, beta 0.9 / 0.999, eps 1e-8) on one batch in
 * device memory (x [n][8], t [n], FP32); asynchronous; *loss_dev (device,
 * optional) receives the batch's loss before the update */
int tp_mlp_train_step_device(tp_mlp* m, const float* x_dev, const float* t_dev, long n, float lr,
                             float* loss_dev);
/* waits for the network's stream; TP_ERR_CUDA if a kernel's tensor-core wait
 * reached its iteration limit */
int tp_mlp_sync(tp_mlp* m);
void* tp_mlp_stream(const tp_mlp* m);
/* C = A B^T on the tensor cores (device pointers, the network's stream): A
 * [M][lda], B [N][ldb] BF16 with K contiguous, C [M][ldc] FP32; M % 128 == 0,
 * N % 32 == 0 with 32 <= N <= 256, K % 64 == 0, lda and ldb multiples of 8 */
int tp_gemm_bf16_device(tp_mlp* m, const void* A, int lda, const void* B, int ldb, float* C, int ldc, int M, int N,
                        int K);

#ifdef __cplusplus
}
#endif
#endif /* THREEPOINT_GB300_H */
