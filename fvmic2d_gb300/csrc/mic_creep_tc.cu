// mic_creep_tc.cu -- tensor-core inference of the creep surrogate (placeholder until the
// tcgen05 kernel lands): routes to an error so callers cannot silently run a CUDA-core path.
#include "mic_internal.cuh"

int mic_creep_surrogate_tc_launch(mic_ctx *ctx, const double *, const double *, const double *, const double *,
                                  int64_t, double *, int *, double *, int *) {
  (void)ctx;
  return MIC_ERR_ARG;
}
