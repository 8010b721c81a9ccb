/*
 * threepoint_gb300 cosmosis module -- the reference's cosmosis entry
 * (cuda_version/interface.cu:16-257) as C functions over a data-block
 * callback table, so that the library has no cosmosis dependency.
 *
 * A cosmosis C++ module forwards its three entry points:
 *   void* setup(cosmosis::DataBlock* o)          -> tp_module_setup(&table_of(o), 0, &m)
 *   DATABLOCK_STATUS execute(DataBlock* b, void* m) -> tp_module_execute(m, &table_of(b))
 *   void cleanup(void* m)                        -> tp_module_cleanup(m)
 * where table_of fills tp_datablock with adapters that call DataBlock::get_val
 * and DataBlock::put_val for the section, key and type each callback names.
 *
 * Keys read and written are the reference's:
 *   setup:   [threepoint] nz_file, zMax, theta_unit, theta_min, theta_max,
 *            theta_bins, diag_only, output_Map3, output_dir   (interface.cu:67-148)
 *   execute: [cosmological_parameters] omega_m, sigma_8, h0, omega_b, n_s, w;
 *            [matter_power_lin] k_h, p_k (first row)          (interface.cu:150-190)
 *            -> [threepoint] Map3s                            (interface.cu:239)
 */
#ifndef THREEPOINT_GB300_MODULE_H
#define THREEPOINT_GB300_MODULE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Data-block access. Every callback returns 0 on success and non-zero when the
 * section/key is missing or has another type. get_string copies at most cap
 * bytes including the terminating zero. get_double_array with buf == NULL only
 * reports the element count in *n; otherwise it copies min(cap, count)
 * elements (a 2-D array such as p_k flattened row-major) and sets *n to count.
 * Booleans (diag_only, output_Map3) are read through get_int. */
typedef struct tp_datablock {
  void* handle;
  int (*get_double)(void* handle, const char* section, const char* key, double* out);
  int (*get_int)(void* handle, const char* section, const char* key, int* out);
  int (*get_string)(void* handle, const char* section, const char* key, char* buf, int cap);
  int (*get_double_array)(void* handle, const char* section, const char* key, double* buf, int cap, int* n);
  int (*put_double_array)(void* handle, const char* section, const char* key, const double* values, int n);
} tp_datablock;

typedef struct tp_module tp_module;

/* setup (interface.cu:67-148): reads the [threepoint] options, the n(z) file
 * (256 bins up to zMax) and builds the aperture-radius triplets: all
 * theta1 <= theta2 <= theta3 of theta_bins log-spaced radii, or only the
 * equal ones if diag_only. The CUDA context on `device` is created by the
 * first execute. Returns a TP_* status; *out is NULL on failure. */
int tp_module_setup(const tp_datablock* options, int device, tp_module** out);

/* execute (interface.cu:150-244): one cosmology per call. Reads the
 * cosmological parameters and the linear P(k) (converted to 256 log bins as
 * convert_Pk, helpers.cu:202-235), builds the tables, evaluates <Map^3> for
 * all triplets in one batch (phi in [0, 2pi], l in [1, 10/theta_min],
 * relative tolerance 1e-4), writes [threepoint] Map3s and, if output_Map3,
 * the file output_dir/om_<om>_sig8_<s8>_h_<h>_w_<w>.dat. */
int tp_module_execute(tp_module* m, const tp_datablock* block);

/* cleanup (interface.cu:251-255) */
int tp_module_cleanup(tp_module* m);

/* No counterpart in the reference: selects TP_FP64 (default) or TP_FP32 for
 * execute; reads the triplets built by setup (out[3 * n] radians). */
int tp_module_set_precision(tp_module* m, int precision);
int tp_module_n_triplets(const tp_module* m);
int tp_module_triplets(const tp_module* m, double* out);
const char* tp_module_last_error(const tp_module* m);

#ifdef __cplusplus
}
#endif
#endif /* THREEPOINT_GB300_MODULE_H */
