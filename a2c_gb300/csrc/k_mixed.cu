// Mixed-precision evaluator (placeholder until the FP32 kernels land).
#include "internal.cuh"

namespace a2c {
a2c_status mixed_eval(a2c_gpp_ctx *, const double *, double *, double *) { return A2C_ERR_INVALID; }
void mixed_free(a2c_gpp_ctx *) {}
}  // namespace a2c
