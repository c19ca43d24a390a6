// a4, precision form: 3xBF16 split covariance on the tcgen05 tensor cores.
#include "common.cuh"

int sg_covariance_tc(sg_handle* h, const float* x, int64_t n_rows, int32_t n_cols, int64_t ld, const float* mu32,
                     const float* sigma32, const uint8_t* row_mask, double* cov, double* zsum, cudaStream_t st) {
  (void)h; (void)x; (void)n_rows; (void)n_cols; (void)ld; (void)mu32; (void)sigma32; (void)row_mask; (void)cov;
  (void)zsum; (void)st;
  return sg::fail(SG_ERR_UNSUPPORTED, "sg_covariance: the precision form is not built yet");
}
