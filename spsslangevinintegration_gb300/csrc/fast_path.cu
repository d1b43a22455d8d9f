// GB300 fast path (placeholder until the fixed-point/FP32 kernels land).
#include "spss_internal.cuh"

namespace spss
{
int fast_create(spss_ctx *) { return SPSS_ERR_NOT_SUPPORTED; }
void fast_destroy(spss_ctx *) {}
int fast_set_state(spss_ctx *, const double *) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_get_state(spss_ctx *, double *) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_evaluate(spss_ctx *, int, const double *, const double *, double *, double, double) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_step(spss_ctx *, int, double, double) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_steps(spss_ctx *, int, double, double, int) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_noise(spss_ctx *, int, unsigned long long, double *) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_complementary_force(spss_ctx *, double *) { return SPSS_ERR_NOT_SUPPORTED; }
int fast_apply_pbc(spss_ctx *) { return SPSS_ERR_NOT_SUPPORTED; }
}  // namespace spss
