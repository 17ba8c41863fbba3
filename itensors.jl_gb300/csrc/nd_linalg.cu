// Blockwise SVD / QR / truncation (placeholder until the batched kernels land).
#include "nd_plan.h"

extern "C" nd_status nd_bs_svd_f64(nd_handle h, int32_t, const int64_t*, const int64_t*, const int64_t*, const double*,
                                   double*, double*, double*, int32_t, int32_t, double, int32_t, int32_t, int32_t,
                                   int32_t*, double*, int32_t*, double*, double*) {
  return nd_fail(h, ND_ERR_UNSUPPORTED, "nd_bs_svd_f64: not built yet");
}
extern "C" nd_status nd_bs_qr_f64(nd_handle h, int32_t, const int64_t*, const int64_t*, const int64_t*, const double*,
                                  double*, double*, int32_t) {
  return nd_fail(h, ND_ERR_UNSUPPORTED, "nd_bs_qr_f64: not built yet");
}
extern "C" nd_status nd_truncate_f64(nd_handle h, const double*, int32_t, int32_t, int32_t, double, int32_t, int32_t,
                                     int32_t*, double*, double*) {
  return nd_fail(h, ND_ERR_UNSUPPORTED, "nd_truncate_f64: not built yet");
}
