// mic_creep_tc.cu -- batch solve of the composite creep law with the surrogate guess from the
// tensor cores (mic_creep_tc.cuh), FP64 Newton polish and exact fallback.
//
// Persistent blocks of 128 threads walk the batch in tiles of 128 samples; each block stages
// the network once, holds 64 TMEM columns for its lifetime and frees them on exit.  At most
// tc::kBlocksPerSM = 5 blocks fit on an SM (about 44 KB of shared memory each), so the 512 TMEM
// columns of an SM are never over-subscribed and an allocation never waits on another block.
#include "mic_creep_tc.cuh"

using namespace mic;

namespace {

__global__ void __launch_bounds__(tc::kTile, tc::kBlocksPerSM) k_creep_surrogate_batch_tc(const double *__restrict__ edot,
                                                                         const double *__restrict__ T,
                                                                         const double *__restrict__ d,
                                                                         const double *__restrict__ P, int64_t n,
                                                                         CreepConfig cfg, double *s_out, int *it_out,
                                                                         double *res_out, int *fb_out,
                                                                         CreepCounters *cc) {
  extern __shared__ unsigned char dyn[];
  tc::Block B;
  tc::setup(B, dyn, cfg.mlp);
  const int64_t ntiles = (n + tc::kTile - 1) / tc::kTile;
#ifndef MIC_EXACT
  const bool coarse = !(cfg.polish_tol < kCoarseTol);  // the polish in double-float arithmetic
#else
  const bool coarse = false;
#endif
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t m = tile * tc::kTile + threadIdx.x;
    const bool valid = m < n;
    double e = 0.0, g = 1.0;
    float f[4] = {0.f, 0.f, 0.f, 0.f}, mref = 0.f;
    CreepCoef k = {1.0, 1.0, 1.0, 1.0};
    CreepTermsDF q;
    bool q_ok = false;
    if (valid) {
      e = edot[m];
      g = grain_arg(d[m]);
#ifndef MIC_EXACT
      if (coarse) {
        q_ok = e > 0.0 && creep_terms_df(T[m], g, P[m], 1.0 / e, q);
        if (q_ok) mref = creep_features_df(q, f);
      } else
#endif
      {
        k = creep_coef(T[m], g, P[m]);
        if (e > 0.0) mref = creep_features(k, e, f);
      }
    }
    const float y = tc::guess(B, f, cfg.tc_wait_limit, &cc->tc_timeouts);
    int it = 0, fb = 0;
    double res = 0.0;
    if (valid) {
      const float lx = creep_guess_lx(cfg.mlp, y, mref);
#ifndef MIC_EXACT
      const double s =
          !coarse ? creep_stress_from_guess(k, e, lx, cfg.tol, cfg.maxit, cfg.polish_iters, cfg.polish_tol, &it,
                                            &res, &fb)
          : e > 0.0 ? creep_stress_coarse(q, q_ok, T[m], g, P[m], e, 1.0 / e, lx, cfg.tol, cfg.maxit,
                                          cfg.polish_iters, cfg.polish_tol, &it, &res, &fb)
                    : 0.0;
#else
      (void)q_ok;
      const double s =
          creep_stress_from_guess(k, e, lx, cfg.tol, cfg.maxit, cfg.polish_iters, cfg.polish_tol, &it, &res, &fb);
#endif
      s_out[m] = s;
      if (it_out) it_out[m] = it;
      if (res_out) res_out[m] = res;
      if (fb_out) fb_out[m] = fb;
    }
    creep_count(cc, valid && e > 0.0, it, res, fb);
  }
  tc::teardown(B, &cc->tc_drain_timeouts);
}

// network outputs for given features (n x 4, row-major) on the tensor-core path
__global__ void __launch_bounds__(tc::kTile, tc::kBlocksPerSM) k_mlp_infer_tc(const float *__restrict__ feat, int64_t n,
                                                             const float *__restrict__ p, float *y_out,
                                                             CreepCounters *cc) {
  extern __shared__ unsigned char dyn[];
  tc::Block B;
  tc::setup(B, dyn, p);
  const int64_t ntiles = (n + tc::kTile - 1) / tc::kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t m = tile * tc::kTile + threadIdx.x;
    float f[4] = {0.f, 0.f, 0.f, 0.f};
    if (m < n)
#pragma unroll
      for (int i = 0; i < 4; ++i) f[i] = feat[4 * m + i];
    const float y = tc::guess(B, f, tc::kWaitLimit, &cc->tc_timeouts);
    if (m < n) y_out[m] = y;
  }
  tc::teardown(B, &cc->tc_drain_timeouts);
}

}  // namespace

int mic_mlp_infer_tc_launch(mic_ctx *ctx, const float *feat, int64_t n, float *y) {
  MIC_CUDA_TRY(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kDynSmem));
  MIC_KERNEL(ctx, "k_mlp_infer_tc");
  k_mlp_infer_tc<<<mic_creep_tc_blocks(ctx, n), tc::kTile, tc::kDynSmem, ctx->stream>>>(feat, n, ctx->mlp, y,
                                                                                         ctx->d_creep);
  return MIC_OK;
}

int mic_creep_tc_blocks(mic_ctx *ctx, int64_t n) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int64_t tiles = (n + tc::kTile - 1) / tc::kTile;
  const int64_t cap = tc::kGridBlocksPerSM * (int64_t)(sms > 0 ? sms : 1);
  return (int)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
}

int mic_creep_surrogate_tc_launch(mic_ctx *ctx, const double *edot, const double *T, const double *d,
                                  const double *P, int64_t n, double *s, int *it, double *res, int *fb) {
  MIC_CUDA_TRY(cudaFuncSetAttribute(k_creep_surrogate_batch_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)tc::kDynSmem));
  MIC_KERNEL(ctx, "k_creep_surrogate_batch_tc");
  k_creep_surrogate_batch_tc<<<mic_creep_tc_blocks(ctx, n), tc::kTile, tc::kDynSmem, ctx->stream>>>(
      edot, T, d, P, n, ctx->creep, s, it, res, fb, ctx->d_creep);
  return MIC_OK;
}
