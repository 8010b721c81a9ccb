// Entry points whose kernels are not yet wired in this build.
#include "tp_capi_internal.h"

extern "C" int tp_pell_batch(tp_ctx* ctx, int, const double*, long, int, double*) {
  return tp_fail(ctx, TP_ERR_STATE, "tp_pell_batch: not available");
}
extern "C" int tp_cov_total_batch(tp_ctx* ctx, int, int, int, double, double, const double*, const double*, int, int,
                                  double*, int*) {
  return tp_fail(ctx, TP_ERR_STATE, "tp_cov_total_batch: not available");
}
