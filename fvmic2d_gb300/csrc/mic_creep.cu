// mic_creep.cu -- the composite ice creep closure (material law 7): exact stress solve, the
// surrogate network's training kernels, and its inference paths.
//
// Surrogate: an MLP 4 -> 64 -> 64 -> 1 with SiLU activations maps normalised
// (log10 edot, T, log10 d, P) to the normalised log10 of the stress s*.  It is trained on the
// GPU by the kernels below on pairs produced by the exact solve, in FP32.  At inference the
// hidden 64x64 layer runs on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in
// tensor memory; mic_creep_tc.cuh); the guess is then polished by FP64 Newton steps and any
// marker still above the residual tolerance finishes with the exact solve in the same thread.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "mic_creep.cuh"
#include "mic_internal.cuh"

using namespace mic;

namespace {

// ---- exact batch solve and training pairs -----------------------------------------------

__global__ void k_creep_exact_batch(const double *edot, const double *T, const double *d, const double *P, int64_t n,
                                    CreepConfig cfg, double *s_out, int *it_out, double *res_out, CreepCounters *cc) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int it = 0, active = 0;
  double res = 0.0;
  if (m < n) {
    const CreepCoef k = creep_coef(T[m], grain_arg(d[m]), P[m]);
    s_out[m] = creep_stress_exact(k, edot[m], cfg.tol, cfg.maxit, &it, &res);
    if (it_out) it_out[m] = it;
    if (res_out) res_out[m] = res;
    active = edot[m] > 0.0;
  }
  creep_count(cc, active, it, res, 0);
}

__device__ __forceinline__ double splitmix_u01(unsigned long long seed, unsigned long long i) {
  unsigned long long z = seed + (i + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// training inputs: log10 edot ~ U[-22,-6] (the workload's U[-18,-10] widened: strain rates of
// stepped markers follow the viscosity and spread further), T ~ U[100,273] K, log10 d ~
// U[-4,-1] m, P ~ U[0, 1e8] Pa; features of their coefficients, target = ln x* - m from the
// exact root of the composite law
__global__ void k_creep_samples(unsigned long long seed, int64_t n, CreepConfig cfg, float *feat, float *target) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const double edot = pow(10.0, -22.0 + 16.0 * splitmix_u01(seed, 4 * m));
  const double T = 100.0 + 173.0 * splitmix_u01(seed, 4 * m + 1);
  const double d = pow(10.0, -4.0 + 3.0 * splitmix_u01(seed, 4 * m + 2));
  const double P = 1e8 * splitmix_u01(seed, 4 * m + 3);
  const CreepCoef k = creep_coef(T, grain_arg(d), P);
  int it;
  double res;
  const double u = creep_root_u(k, edot, cfg.tol, cfg.maxit, &it, &res);
  float f[4];
  const float mref = creep_features(k, edot, f);
#pragma unroll
  for (int i = 0; i < 4; ++i) feat[4 * m + i] = f[i];
  target[m] = (float)(u - kLn1e6 - (double)mref);
}

// ---- training: per-block forward/backward with deterministic partial gradients -------

constexpr int kTB = 128;  // samples per block

// Loss = mean over the batch of (y - t)^2 with t = (log10 s - out_mu) / out_sigma.
// part[block][kNTrain] receives the block's gradient sums; lpart[block] its loss sum.
__global__ void __launch_bounds__(kTB) k_train_fwdbwd(const float *__restrict__ p, const float *__restrict__ feat,
                                                      const float *__restrict__ target,
                                                      const int *__restrict__ index, int64_t nb, float inv_batch,
                                                      float *__restrict__ part, float *__restrict__ lpart) {
  extern __shared__ float sm[];
  float *w2s = sm;                    // 64*64
  float *h1s = w2s + kH * kH;         // [128][64]
  float *h2s = h1s + kTB * kH;        // [128][64]
  float *dz2s = h2s + kTB * kH;       // [128][64]
  float *dz1s = dz2s + kTB * kH;      // [128][64]
  float *fs = dz1s + kTB * kH;        // [128][4]
  float *dys = fs + kTB * 4;          // [128]
  const int t = threadIdx.x;
  for (int q = t; q < kH * kH; q += kTB) w2s[q] = bf16_round(p[kOffW2 + q]);
  const int64_t b = (int64_t)blockIdx.x * kTB + t;
  const bool valid = b < nb;
  const int s = valid ? index[b] : 0;
  float f[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) f[i] = valid ? feat[4 * (int64_t)s + i] : 0.0f;
  __syncthreads();
  // forward, keeping pre-activations for the backward pass
  float z1[kH], h1[kH];
#pragma unroll
  for (int n = 0; n < kH; ++n) {
    float z = p[kOffB1 + n];
#pragma unroll
    for (int i = 0; i < 4; ++i) z = fmaf(p[kOffW1 + 4 * n + i], f[i], z);
    z1[n] = z;
    h1[n] = silu(z);
    h1s[t * kH + n] = h1[n];
  }
  float y = p[kOffB3];
  for (int n = 0; n < kH; ++n) {
    float z = p[kOffB2 + n];
#pragma unroll 16
    for (int k = 0; k < kH; ++k) z = fmaf(w2s[n * kH + k], h1[k], z);
    const float h2 = silu(z);
    h2s[t * kH + n] = h2;
    dz2s[t * kH + n] = z;  // pre-activation for now
    y = fmaf(p[kOffW3 + n], h2, y);
  }
  const float tt = valid ? (target[s] - p[kOffNorm]) / p[kOffNorm + 1] : 0.0f;
  const float err = valid ? (y - tt) : 0.0f;
  const float dy = 2.0f * err * inv_batch;
  dys[t] = dy;
  // backward through layer 3 and the second activation
  for (int n = 0; n < kH; ++n) {
    const float z = dz2s[t * kH + n];
    dz2s[t * kH + n] = dy * p[kOffW3 + n] * dsilu(z);
  }
  // dh1 = W2^T dz2, then through the first activation
#pragma unroll 4
  for (int k = 0; k < kH; ++k) {
    float acc = 0.0f;
    for (int n = 0; n < kH; ++n) acc = fmaf(w2s[n * kH + k], dz2s[t * kH + n], acc);
    dz1s[t * kH + k] = acc * dsilu(z1[k]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) fs[t * 4 + i] = f[i];
  __syncthreads();
  // block partial gradients, each summed over the block's samples in index order
  float *g = part + (size_t)blockIdx.x * kNTrain;
  for (int q = t; q < kH * kH; q += kTB) {  // dW2[n][k] = sum dz2[n] h1[k]
    const int n = q / kH, k = q % kH;
    float acc = 0.0f;
    for (int r = 0; r < kTB; ++r) acc = fmaf(dz2s[r * kH + n], h1s[r * kH + k], acc);
    g[kOffW2 + q] = acc;
  }
  for (int q = t; q < kH * 4; q += kTB) {  // dW1[n][i] = sum dz1[n] f[i]
    const int n = q / 4, i = q % 4;
    float acc = 0.0f;
    for (int r = 0; r < kTB; ++r) acc = fmaf(dz1s[r * kH + n], fs[r * 4 + i], acc);
    g[kOffW1 + q] = acc;
  }
  if (t < kH) {
    float a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int r = 0; r < kTB; ++r) {
      a1 += dz1s[r * kH + t];
      a2 += dz2s[r * kH + t];
      a3 = fmaf(dys[r], h2s[r * kH + t], a3);
    }
    g[kOffB1 + t] = a1;
    g[kOffB2 + t] = a2;
    g[kOffW3 + t] = a3;
  }
  if (t == 0) {
    float a = 0.0f;
    for (int r = 0; r < kTB; ++r) a += dys[r];
    g[kOffB3] = a;
  }
  // loss partial: warp shuffles then one value per block
  float l = err * err;
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  __shared__ float lw[kTB / 32];
  if ((t & 31) == 0) lw[t >> 5] = l;
  __syncthreads();
  if (t == 0) {
    float a = 0.0f;
    for (int w = 0; w < kTB / 32; ++w) a += lw[w];
    lpart[blockIdx.x] = a;
  }
}

// gradient = sum of the block partials in block order; optional Adam step
__global__ void k_train_reduce(float *p, const float *part, int nblocks, float *grad, float *m_, float *v_, int step,
                               float lr, int apply) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kNTrain) return;
  float g = 0.0f;
  for (int b = 0; b < nblocks; ++b) g += part[(size_t)b * kNTrain + q];
  if (grad) grad[q] = g;
  if (!apply) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float m = b1 * m_[q] + (1.0f - b1) * g;
  const float v = b2 * v_[q] + (1.0f - b2) * g * g;
  m_[q] = m;
  v_[q] = v;
  const float mh = m / (1.0f - powf(b1, (float)step));
  const float vh = v / (1.0f - powf(b2, (float)step));
  p[q] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_sum_floats(const float *a, int n, float *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float s = 0.0f;
  for (int i = 0; i < n; ++i) s += a[i];
  *out = s;
}

// deterministic shuffle of sample indices for one epoch: the affine permutation
// i -> (a i + c) mod n, with a coprime to n chosen on the host
__global__ void k_epoch_order(int *idx, int64_t n, unsigned long long a, unsigned long long c) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  idx[i] = (int)((a * (unsigned long long)i + c) % (unsigned long long)n);
}

// ---- surrogate batch inference (FP32 CUDA cores) + polish + fallback ------------------

__global__ void __launch_bounds__(128) k_creep_surrogate_batch_fp32(const double *edot, const double *T,
                                                                     const double *d, const double *P, int64_t n,
                                                                     CreepConfig cfg, double *s_out, int *it_out,
                                                                     double *res_out, int *fb_out,
                                                                     CreepCounters *cc) {
  __shared__ float w2s[kH * kH];
  for (int q = threadIdx.x; q < kH * kH; q += blockDim.x) w2s[q] = bf16_round(cfg.mlp[kOffW2 + q]);
  __syncthreads();
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int it = 0, fb = 0, active = 0;
  double res = 0.0;
  if (m < n) {
    const double e = edot[m], g = grain_arg(d[m]);
#ifndef MIC_EXACT
    if (!(cfg.polish_tol < kCoarseTol)) {  // the polish in double-float arithmetic
      CreepTermsDF q;
      const bool q_ok = e > 0.0 && creep_terms_df(T[m], g, P[m], 1.0 / e, q);
      float lx0 = 0.f;
      if (q_ok && !(q.a.hi > 1e6f)) {  // the network is consulted on the non-linear branch only
        float f[4];
        const float mref = creep_features_df(q, f);
        lx0 = creep_guess_lx(cfg.mlp, mlp_forward(cfg.mlp, w2s, f), mref);
      }
      s_out[m] = e > 0.0 ? creep_stress_coarse(q, q_ok, T[m], g, P[m], e, 1.0 / e, lx0, cfg.tol, cfg.maxit,
                                               cfg.polish_iters, cfg.polish_tol, &it, &res, &fb)
                         : 0.0;
    } else
#endif
    {
    const CreepCoef k = creep_coef(T[m], g, P[m]);
    float lx0 = 0.f;
    if (e > 0.0 && e / k.C >= 1.0) {  // the network is consulted on the non-linear branch only
      float f[4];
      const float mref = creep_features(k, e, f);
      lx0 = creep_guess_lx(cfg.mlp, mlp_forward(cfg.mlp, w2s, f), mref);
    }
    s_out[m] = creep_stress_from_guess(k, e, lx0, cfg.tol, cfg.maxit, cfg.polish_iters, cfg.polish_tol, &it, &res,
                                       &fb);
    }
    if (it_out) it_out[m] = it;
    if (res_out) res_out[m] = res;
    if (fb_out) fb_out[m] = fb;
    active = e > 0.0;
  }
  creep_count(cc, active, it, res, fb);
}

__global__ void __launch_bounds__(128) k_mlp_infer_fp32(const float *__restrict__ feat, int64_t n,
                                                         const float *__restrict__ p, float *y_out) {
  __shared__ float w2s[kH * kH];
  for (int q = threadIdx.x; q < kH * kH; q += blockDim.x) w2s[q] = bf16_round(p[kOffW2 + q]);
  __syncthreads();
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  float f[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) f[i] = feat[4 * m + i];
  y_out[m] = mlp_forward(p, w2s, f);
}

// He-style uniform initialisation from SplitMix64 (deterministic)
__global__ void k_mlp_init(float *p, unsigned long long seed) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= kNParams) return;
  const float u = (float)(2.0 * splitmix_u01(seed, q) - 1.0);
  float v = 0.0f;
  if (q < kOffB1)
    v = u * 1.2247449f;  // sqrt(6 / 4)
  else if (q >= kOffW2 && q < kOffB2)
    v = u * 0.30618622f;  // sqrt(6 / 64)
  else if (q >= kOffW3 && q < kOffB3)
    v = u * 0.30618622f;
  p[q] = v;
}

int ensure_train(mic_ctx *ctx, int64_t floats) {
  if (ctx->train_cap >= floats) return MIC_OK;
  cudaFree(ctx->train_buf);
  ctx->train_buf = nullptr;
  ctx->train_cap = 0;
  if (cudaMalloc((void **)&ctx->train_buf, sizeof(float) * floats) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->train_cap = floats;
  return MIC_OK;
}

int ensure_mlp(mic_ctx *ctx) {
  if (ctx->mlp) return MIC_OK;
  if (cudaMalloc((void **)&ctx->mlp, sizeof(float) * kNParams) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->creep.mlp = ctx->mlp;
  ctx->gen++;
  return MIC_OK;
}

size_t fwdbwd_smem() { return sizeof(float) * (kH * kH + 4 * kTB * kH + kTB * 4 + kTB); }

// W2 of a host copy of the parameters rounded to BF16 (round to nearest even, as
// __float2bfloat16_rn; the weights are finite)
void round_w2_bf16(float *p) {
  for (int q = kOffW2; q < kOffB2; ++q) {
    uint32_t u;
    memcpy(&u, &p[q], sizeof(u));
    if ((u & 0x7F800000u) == 0x7F800000u) continue;
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    memcpy(&p[q], &u, sizeof(u));
  }
}

// content key of a network's parameters (FNV-1a over their bytes, never 0): contexts whose keys
// agree hold the same network, so a batch of their marker passes may read any one of the copies
unsigned long long net_key(const float *p) {
  const unsigned char *b = reinterpret_cast<const unsigned char *>(p);
  unsigned long long h = 1469598103934665603ULL;
  for (size_t i = 0; i < sizeof(float) * kNParams; ++i) h = (h ^ b[i]) * 1099511628211ULL;
  return h ? h : 1ULL;
}

}  // namespace

// grain sizes -> the grain argument the creep coefficients take (grain_arg), in place
__global__ void k_grain_arg(double *g, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < n) g[m] = grain_arg(g[m]);
}

// ---- C ABI ---------------------------------------------------------------------------

extern "C" int mic_creep_param_count(void) { return kNParams; }

extern "C" int mic_creep_configure(mic_ctx *ctx, int mode, double tol, int maxit, int polish_iters,
                                   double polish_tol) {
  if (!ctx || mode < 0 || mode > 2 || !(tol > 0.0) || maxit < 1 || maxit > 1000 || polish_iters < 0 ||
      polish_iters > 50 || !(polish_tol > 0.0))
    return MIC_ERR_ARG;
  if (mode >= 1 && !ctx->mlp) return MIC_ERR_ARG;
  ctx->creep.mode = mode;
  ctx->creep.tol = tol;
  ctx->creep.maxit = maxit;
  ctx->creep.polish_iters = polish_iters;
  ctx->creep.polish_tol = polish_tol;
  ctx->gen++;
  return MIC_OK;
}

// Limit of the bounded wait on each tensor-core tile's completion barrier (try_wait rounds;
// default 2^20).  A tile whose wait runs out makes its block stop using the tensor cores; its
// markers take the exact solve, and mic_creep_tc_stats counts it.
extern "C" int mic_creep_set_tc_wait_limit(mic_ctx *ctx, int rounds) {
  if (!ctx || rounds < 0) return MIC_ERR_ARG;
  ctx->creep.tc_wait_limit = rounds;
  ctx->gen++;
  return MIC_OK;
}

extern "C" int mic_creep_tc_stats(mic_ctx *ctx, int64_t *tile_timeouts, int64_t *drain_timeouts) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  CreepCounters h;
  MIC_CUDA_TRY(cudaMemcpyAsync(&h, ctx->d_creep, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (tile_timeouts) *tile_timeouts = (int64_t)h.tc_timeouts;
  if (drain_timeouts) *drain_timeouts = (int64_t)h.tc_drain_timeouts;
  return MIC_OK;
}

extern "C" int mic_markers_set_grain_size(mic_ctx *ctx, const double *d, int64_t n) {
  if (!ctx || !d || n != ctx->n) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n == 0) return MIC_OK;
  // grain sizes arrive in the caller's order; the columns are in device order: scatter by id
  double *tmp = ctx->scr0;
  MIC_CUDA_TRY(cudaMemcpyAsync(tmp, d, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int e = mic_gather_by_id(ctx, tmp, ctx->f64[C_GRAIN]);
  if (e) return e;
  MIC_KERNEL(ctx, "k_grain_arg");
  k_grain_arg<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->f64[C_GRAIN], n);
  ctx->has_grain = 1;
  ctx->gen++;
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_creep_set_mlp(mic_ctx *ctx, const float *params, int n) {
  if (!ctx || !params || n != kNParams) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  int e = ensure_mlp(ctx);
  if (e) return e;
  std::vector<float> h(params, params + kNParams);
  round_w2_bf16(h.data());
  MIC_CUDA_TRY(cudaMemcpyAsync(ctx->mlp, h.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->mlp_key = net_key(h.data());
  ctx->gen++;  // captured steps may read this network through another context's copy
  return MIC_OK;
}

extern "C" int mic_creep_get_mlp(mic_ctx *ctx, float *params, int n) {
  if (!ctx || !params || n != kNParams || !ctx->mlp) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaMemcpyAsync(params, ctx->mlp, sizeof(float) * kNParams, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// Solve a batch of (edot, T, d, P) held in host arrays: mode 0 exact, 1 surrogate (FP32
// CUDA-core inference), 2 surrogate with tensor-core inference.  Outputs: stress, iterations,
// final residual |rate/edot - 1| and fallback flags (any output may be NULL).
extern "C" int mic_creep_solve_batch(mic_ctx *ctx, const double *edot, const double *T, const double *d,
                                     const double *P, int64_t n, int mode, double *s_out, int32_t *it_out,
                                     double *res_out, int32_t *fb_out) {
  if (!ctx || n < 0 || !edot || !T || !d || !P || !s_out || mode < 0 || mode > 2) return MIC_ERR_ARG;
  if ((mode >= 1) && !ctx->mlp) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n == 0) return MIC_OK;
  // device staging in the training buffer: 4 inputs + s + res (doubles) + it + fb (ints)
  const int64_t need = n * (2 * 6 + 2);
  int e = ensure_train(ctx, need);
  if (e) return e;
  double *db = reinterpret_cast<double *>(ctx->train_buf);
  double *de = db, *dT = db + n, *dd = db + 2 * n, *dP = db + 3 * n, *ds = db + 4 * n, *dr = db + 5 * n;
  int *di = reinterpret_cast<int *>(db + 6 * n), *df = di + n;
  MIC_CUDA_TRY(cudaMemcpyAsync(de, edot, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(dT, T, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(dd, d, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(dP, P, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(df, 0, sizeof(int) * n, ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(ctx->d_creep, 0, sizeof(CreepCounters), ctx->stream));
  if (mode == 0) {
    MIC_KERNEL(ctx, "k_creep_exact_batch");
    k_creep_exact_batch<<<grid_for(n), kBlock, 0, ctx->stream>>>(de, dT, dd, dP, n, ctx->creep, ds, di, dr,
                                                                 ctx->d_creep);
  } else if (mode == 1) {
    MIC_KERNEL(ctx, "k_creep_surrogate_batch_fp32");
    k_creep_surrogate_batch_fp32<<<grid_for(n, 128), 128, 0, ctx->stream>>>(de, dT, dd, dP, n, ctx->creep, ds, di,
                                                                           dr, df, ctx->d_creep);
  } else {
    e = mic_creep_surrogate_tc_launch(ctx, de, dT, dd, dP, n, ds, di, dr, df);
    if (e) return e;
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(s_out, ds, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (it_out) MIC_CUDA_TRY(cudaMemcpyAsync(it_out, di, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (res_out) MIC_CUDA_TRY(cudaMemcpyAsync(res_out, dr, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (fb_out) MIC_CUDA_TRY(cudaMemcpyAsync(fb_out, df, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// Network outputs y[n] for features feat[n][4] (host arrays) with the context's parameters:
// mode 1 on the CUDA cores in FP32, mode 2 with the hidden layer on the tensor cores.
extern "C" int mic_creep_mlp_infer(mic_ctx *ctx, const float *feat, int64_t n, int mode, float *y) {
  if (!ctx || !feat || !y || n < 0 || mode < 1 || mode > 2 || !ctx->mlp) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n == 0) return MIC_OK;
  int e = ensure_train(ctx, 5 * n);
  if (e) return e;
  float *df = ctx->train_buf, *dy = df + 4 * n;
  MIC_CUDA_TRY(cudaMemcpyAsync(df, feat, sizeof(float) * 4 * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(ctx->d_creep, 0, sizeof(CreepCounters), ctx->stream));
  if (mode == 1) {
    MIC_KERNEL(ctx, "k_mlp_infer_fp32");
    k_mlp_infer_fp32<<<grid_for(n, 128), 128, 0, ctx->stream>>>(df, n, ctx->mlp, dy);
  } else if ((e = mic_mlp_infer_tc_launch(ctx, df, n, dy))) {
    return e;
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// Gradient of the mean squared loss over n samples (n a multiple of 128) at the given
// parameters, from the training kernels: grad[kNParams-2] (normalisation excluded), *loss.
extern "C" int mic_creep_mlp_grad(mic_ctx *ctx, const float *params, const float *feat, const float *target,
                                  int n, float *grad, float *loss) {
  if (!ctx || !params || !feat || !target || !grad || n <= 0 || n % kTB) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int nblocks = n / kTB;
  // params, features (4n), targets (n), sample order (n ints), partials, loss partials, gradient, loss
  const int64_t need = (int64_t)kNParams + 6 * (int64_t)n + (int64_t)nblocks * kNTrain + nblocks + kNTrain + 8;
  int e = ensure_train(ctx, need);
  if (e) return e;
  float *p = ctx->train_buf, *fe = p + kNParams, *tg = fe + 4 * (int64_t)n;
  int *ix = reinterpret_cast<int *>(tg + n);
  float *part = reinterpret_cast<float *>(ix + n), *lp = part + (size_t)nblocks * kNTrain, *g = lp + nblocks;
  float *ls = g + kNTrain;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  MIC_CUDA_TRY(cudaMemcpyAsync(p, params, sizeof(float) * kNParams, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(fe, feat, sizeof(float) * 4 * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(tg, target, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(ix, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaFuncSetAttribute(k_train_fwdbwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwdbwd_smem()));
  {
    MIC_KERNEL(ctx, "k_train_fwdbwd");
    k_train_fwdbwd<<<nblocks, kTB, fwdbwd_smem(), ctx->stream>>>(p, fe, tg, ix, n, 1.0f / n, part, lp);
  }
  {
    MIC_KERNEL(ctx, "k_train_reduce");
    k_train_reduce<<<(kNTrain + 255) / 256, 256, 0, ctx->stream>>>(p, part, nblocks, g, nullptr, nullptr, 0, 0.f,
                                                                   0);
  }
  {
    MIC_KERNEL(ctx, "k_sum_floats");
    k_sum_floats<<<1, 32, 0, ctx->stream>>>(lp, nblocks, ls);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(grad, g, sizeof(float) * kNTrain, cudaMemcpyDeviceToHost, ctx->stream));
  float l = 0.f;
  MIC_CUDA_TRY(cudaMemcpyAsync(&l, ls, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = l / n;
  return MIC_OK;
}

// Train the context's surrogate on GPU-generated pairs: nsamples exact solves from the workload
// distribution (seed), then `steps` Adam steps on minibatches of `batch` (multiple of 128) with a
// cosine learning-rate decay from lr.  loss_hist[steps] (optional) receives the batch losses.
extern "C" int mic_creep_train(mic_ctx *ctx, int64_t nsamples, int batch, int steps, float lr,
                               unsigned long long seed, float *loss_hist) {
  if (!ctx || nsamples < batch || batch <= 0 || batch % kTB || steps <= 0 || !(lr > 0.f) ||
      nsamples > (int64_t)1 << 28)
    return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  int e = ensure_mlp(ctx);
  if (e) return e;
  ctx->mlp_key = 0;  // the network is rewritten below
  const int nblocks = batch / kTB;
  // features (4n), targets (n), sample order (n ints), partials, loss partials, Adam moments, losses
  const int64_t need = 6 * nsamples + (int64_t)nblocks * kNTrain + nblocks + 2 * (int64_t)kNTrain + steps + 16;
  if ((e = ensure_train(ctx, need))) return e;
  float *fe = ctx->train_buf, *tg = fe + 4 * nsamples;
  int *ix = reinterpret_cast<int *>(tg + nsamples);
  float *part = reinterpret_cast<float *>(ix + nsamples), *lp = part + (size_t)nblocks * kNTrain;
  float *am = lp + nblocks, *av = am + kNTrain, *lh = av + kNTrain;
  {
    MIC_KERNEL(ctx, "k_creep_samples");
    k_creep_samples<<<grid_for(nsamples), kBlock, 0, ctx->stream>>>(seed, nsamples, ctx->creep, fe, tg);
  }
  // output normalisation from the targets (host: mean and spread of log10 s*)
  std::vector<float> ht(nsamples);
  MIC_CUDA_TRY(cudaMemcpyAsync(ht.data(), tg, sizeof(float) * nsamples, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  double mu = 0.0, sq = 0.0;
  for (int64_t i = 0; i < nsamples; ++i) mu += ht[i];
  mu /= nsamples;
  for (int64_t i = 0; i < nsamples; ++i) sq += (ht[i] - mu) * (ht[i] - mu);
  const float norm[2] = {(float)mu, (float)std::sqrt(sq / nsamples)};
  {
    MIC_KERNEL(ctx, "k_mlp_init");
    k_mlp_init<<<(kNParams + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp, seed ^ 0x5DEECE66DULL);
  }
  MIC_CUDA_TRY(cudaMemcpyAsync(ctx->mlp + kOffNorm, norm, sizeof(norm), cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaMemsetAsync(am, 0, sizeof(float) * 2 * kNTrain, ctx->stream));
  MIC_CUDA_TRY(cudaFuncSetAttribute(k_train_fwdbwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwdbwd_smem()));
  const int64_t per_epoch = nsamples / batch;
  for (int s = 0; s < steps; ++s) {
    const int epoch = (int)(s / per_epoch);
    if (s % per_epoch == 0) {
      unsigned long long a = (2654435761ULL * (2ULL * (unsigned long long)epoch + 1ULL) + seed) % (unsigned long long)nsamples;
      while (a == 0 || std::gcd(a, (unsigned long long)nsamples) != 1ULL) a = (a + 1) % (unsigned long long)nsamples;
      const unsigned long long c = (7919ULL * (unsigned long long)epoch + seed) % (unsigned long long)nsamples;
      MIC_KERNEL(ctx, "k_epoch_order");
      k_epoch_order<<<grid_for(nsamples), kBlock, 0, ctx->stream>>>(ix, nsamples, a, c);
    }
    const int64_t off = (s % per_epoch) * (int64_t)batch;
    {
      MIC_KERNEL(ctx, "k_train_fwdbwd");
      k_train_fwdbwd<<<nblocks, kTB, fwdbwd_smem(), ctx->stream>>>(ctx->mlp, fe, tg, ix + off, batch, 1.0f / batch,
                                                                    part, lp);
    }
    const float lrs = 0.5f * lr * (1.0f + cosf(3.14159265f * s / steps));
    {
      MIC_KERNEL(ctx, "k_train_reduce");
      k_train_reduce<<<(kNTrain + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp, part, nblocks, nullptr, am, av, s + 1,
                                                                     lrs, 1);
    }
    {
      MIC_KERNEL(ctx, "k_sum_floats");
      k_sum_floats<<<1, 32, 0, ctx->stream>>>(lp, nblocks, lh + s);
    }
  }
  MIC_CUDA_TRY(cudaGetLastError());
  if (loss_hist) {
    MIC_CUDA_TRY(cudaMemcpyAsync(loss_hist, lh, sizeof(float) * steps, cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (int s = 0; s < steps; ++s) loss_hist[s] /= batch;
  }
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  {
    // the trained FP32 master of W2 rounded to the BF16 values the forward passes used
    std::vector<float> h(kNParams);
    MIC_CUDA_TRY(cudaMemcpy(h.data(), ctx->mlp, sizeof(float) * kNParams, cudaMemcpyDeviceToHost));
    round_w2_bf16(h.data());
    MIC_CUDA_TRY(cudaMemcpy(ctx->mlp, h.data(), sizeof(float) * kNParams, cudaMemcpyHostToDevice));
    ctx->mlp_key = net_key(h.data());
  }
  ctx->creep.mlp = ctx->mlp;
  ctx->gen++;
  return MIC_OK;
}

// creep counters of the last rheology pass
extern "C" int mic_creep_stats(mic_ctx *ctx, int64_t *markers, int64_t *iterations, int64_t *fallbacks,
                               double *max_residual, int64_t *tc_timeouts) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  CreepCounters h;
  MIC_CUDA_TRY(cudaMemcpyAsync(&h, ctx->d_creep, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (markers) *markers = (int64_t)h.markers;
  if (iterations) *iterations = (int64_t)h.iterations;
  if (fallbacks) *fallbacks = (int64_t)h.fallbacks;
  if (max_residual) memcpy(max_residual, &h.max_res_bits, sizeof(double));
  if (tc_timeouts) *tc_timeouts = (int64_t)h.tc_timeouts;
  return MIC_OK;
}

// ---- the closure's exports under their short names (exact solve, training, inference) --------

// exact composite-creep Newton solve of a host batch (mic_creep_solve_batch, mode 0)
extern "C" int mic_creep_newton(mic_ctx *ctx, const double *edot, const double *T, const double *d,
                                const double *P, int64_t n, double *stress, int32_t *iterations, double *residual) {
  return mic_creep_solve_batch(ctx, edot, T, d, P, n, 0, stress, iterations, residual, nullptr);
}

extern "C" int mic_surrogate_train(mic_ctx *ctx, int64_t nsamples, int batch, int steps, float lr,
                                   unsigned long long seed, float *loss_hist) {
  return mic_creep_train(ctx, nsamples, batch, steps, lr, seed, loss_hist);
}

extern "C" int mic_surrogate_infer(mic_ctx *ctx, const float *feat, int64_t n, int mode, float *y) {
  return mic_creep_mlp_infer(ctx, feat, n, mode, y);
}
