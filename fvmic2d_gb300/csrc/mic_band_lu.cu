// mic_band_lu.cu -- direct solve of an assembled system on the device: LU factorisation with
// partial pivoting of the banded matrix, then the triangular solves.  It stands in for
// kspLinearSolve (kspLinearSolve.c:13-120) run as the reference's option files configure it,
// `-stokes_ksp_type preonly -stokes_pc_type lu` and the same for `energy_`
// (option_files/run_mumps.petscopt), i.e. one direct factorisation and solve per call.
//
// Ordering: the staggered stencils couple a node to its 8 neighbours, so numbering the nodes
// along the shorter grid direction first gives a band of about dof (min(NX, NY) + 1) on each
// side.  The matrix goes into row-band storage, row i holding columns i-kl .. i+kl+ku (the extra
// kl for the fill that row interchanges bring), W = 2 kl + ku + 1 values per row.
//
// Factorisation, right-looking in panels of NB columns:
//   panel  one CTA: the panel's (NB + kl) x NB block in shared memory, column by column: pivot
//          row (largest |value|, first on ties), interchange (whole rows, the right-hand side
//          too), multipliers, rank-1 update of the panel; the forward substitution of the
//          right-hand side rides along (it is one more column);
//   trsm   U12 = L11^-1 A12 for the columns right of the panel, one thread per column;
//   update A22 -= L21 U12 over the band window, 64 x 64 tiles.
// Interchanges inside a panel move whole panel rows, multipliers included, so that the panel's
// L is in final row order for the deferred trsm and update; interchanges can carry multipliers
// outside the band, so the panel's L goes to a dense (NB + kl) x NB buffer rather than back into
// the band, which keeps only U.  Back substitution: one CTA, 32 rows at a time (a warp per row
// for the part from solved unknowns, one warp for the triangle).
#include <algorithm>
#include <climits>
#include <cmath>

#include "mic_internal.cuh"

using namespace mic;

namespace {

__device__ __forceinline__ int64_t bmap(int64_t r, int dof, int NX, int NY, int transpose) {
  if (!transpose) return r;
  const int64_t node = r / dof;
  const int d = (int)(r % dof);
  const int ix = (int)(node % NX), jy = (int)(node / NX);
  return ((int64_t)ix * NY + jy) * dof + d;
}

__global__ void k_band_width(const int *__restrict__ cnt, const int *__restrict__ col, int width, int64_t n,
                             int dof, int NX, int NY, int transpose, int *bw) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t bi = bmap(r, dof, NX, NY, transpose);
  int lo = 0, up = 0;
  for (int k = 0; k < cnt[r]; ++k) {
    const int64_t bj = bmap(col[r * width + k], dof, NX, NY, transpose);
    lo = max(lo, (int)(bi - bj));
    up = max(up, (int)(bj - bi));
  }
  atomicMax(&bw[0], lo);
  atomicMax(&bw[1], up);
}

__global__ void k_band_scatter(const int *__restrict__ cnt, const int *__restrict__ col,
                               const double *__restrict__ val, const double *__restrict__ rhs, int width, int64_t n,
                               int dof, int NX, int NY, int transpose, int kl, int W, double *band, double *b) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t bi = bmap(r, dof, NX, NY, transpose);
  for (int k = 0; k < cnt[r]; ++k) {
    const int64_t bj = bmap(col[r * width + k], dof, NX, NY, transpose);
    band[bi * W + (bj - bi + kl)] = val[r * width + k];
  }
  b[bi] = rhs[r];
}

__global__ void k_band_gather(const double *__restrict__ x, int64_t n, int dof, int NX, int NY, int transpose,
                              double *out) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r < n) out[r] = x[bmap(r, dof, NX, NY, transpose)];
}

constexpr int kPanelThreads = 1024;

template <int NB>
__global__ void __launch_bounds__(kPanelThreads) k_band_panel(double *band, int64_t n, int kl, int ku, int W,
                                                             int64_t k0, int *piv, double *b, int *info,
                                                             double *Lbuf) {
  extern __shared__ double sp[];  // [R][NB]
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  __shared__ int s_p;
  __shared__ double s_bj;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  const int R = (int)(min(n, k1 + kl) - k0);
  for (int idx = tid; idx < R * NB; idx += blockDim.x) {
    const int r = idx / NB, c = idx % NB;
    const int off = c - r + kl;
    sp[idx] = (c < nbc && off >= 0 && off < W) ? band[(k0 + r) * (int64_t)W + off] : 0.0;
  }
  __syncthreads();
  for (int jj = 0; jj < nbc; ++jj) {
    const int64_t j = k0 + jj;
    const int rmax = (int)(min(n - 1, j + kl) - k0);
    // pivot: largest |a|, the first of equal ones (LAPACK's idamax)
    double bv = -1.0;
    int bi = INT_MAX;
    for (int r = jj + tid; r <= rmax; r += blockDim.x) {
      const double a = fabs(sp[r * NB + jj]);
      if (a > bv) {
        bv = a;
        bi = r;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_down_sync(0xffffffffu, bv, o);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
      if (v2 > bv || (v2 == bv && i2 < bi)) {
        bv = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      red_v[warp] = bv;
      red_i[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      bv = lane < nwarps ? red_v[lane] : -1.0;
      bi = lane < nwarps ? red_i[lane] : INT_MAX;
      for (int o = 16; o > 0; o >>= 1) {
        const double v2 = __shfl_down_sync(0xffffffffu, bv, o);
        const int i2 = __shfl_down_sync(0xffffffffu, bi, o);
        if (v2 > bv || (v2 == bv && i2 < bi)) {
          bv = v2;
          bi = i2;
        }
      }
      if (lane == 0) s_p = (bi >= jj && bi <= rmax) ? bi : jj;  // all NaN: keep the diagonal
    }
    __syncthreads();
    const int p = s_p;
    if (p != jj) {
      // whole panel rows: the multipliers of earlier columns move with their rows, so that the
      // panel's L is in final row order for the deferred update
      for (int c = tid; c < NB; c += blockDim.x) {
        const double t = sp[jj * NB + c];
        sp[jj * NB + c] = sp[p * NB + c];
        sp[p * NB + c] = t;
      }
      const int64_t q = k0 + p;
      const int64_t cend = min(n - 1, j + kl + ku);
      for (int64_t c = k1 + tid; c <= cend; c += blockDim.x) {
        double *a = band + j * W + (c - j + kl);
        double *bq = band + q * W + (c - q + kl);
        const double t = *a;
        *a = *bq;
        *bq = t;
      }
      if (tid == 0) {
        const double t = b[j];
        b[j] = b[q];
        b[q] = t;
      }
    }
    if (tid == 0) piv[j] = (int)(k0 + p);
    __syncthreads();
    if (tid == 0) s_bj = b[j];
    const double d = sp[jj * NB + jj];
    if (d == 0.0 && tid == 0) atomicMin(info, (int)j);
    __syncthreads();
    const double bj = s_bj;
    if (d != 0.0) {
      for (int r = jj + 1 + tid; r <= rmax; r += blockDim.x) {
        const double l = sp[r * NB + jj] / d;
        sp[r * NB + jj] = l;
        b[k0 + r] -= l * bj;
      }
    }
    __syncthreads();
    const int ncol = nbc - 1 - jj, nrow = rmax - jj;
    for (int idx = tid; idx < nrow * ncol; idx += blockDim.x) {
      const int r = jj + 1 + idx / ncol, c = jj + 1 + idx % ncol;
      sp[r * NB + c] -= sp[r * NB + jj] * sp[jj * NB + c];
    }
    __syncthreads();
  }
  // U of the panel rows back into the band; the whole panel (L11 and L21, which row
  // interchanges can carry outside the band) to the dense panel buffer
  for (int idx = tid; idx < R * NB; idx += blockDim.x) {
    const int r = idx / NB, c = idx % NB;
    const int off = c - r + kl;
    if (c < nbc && c >= r && off < W) band[(k0 + r) * (int64_t)W + off] = sp[idx];
    Lbuf[idx] = sp[idx];
  }
}

// U12 = L11^-1 A12: columns k1 .. k1 + ncols - 1, one thread each
template <int NB>
__global__ void k_band_trsm(double *band, int64_t n, int kl, int W, int64_t k0, int ncols,
                            const double *__restrict__ Lbuf) {
  __shared__ double L[NB][NB];
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int ii = idx / NB, jj = idx % NB;
    L[ii][jj] = (ii > jj && ii < nbc) ? Lbuf[idx] : 0.0;
  }
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncols) return;
  const int64_t c = k1 + t;
  double u[NB];
#pragma unroll
  for (int ii = 0; ii < NB; ++ii) {
    const int64_t off = c - (k0 + ii) + kl;
    u[ii] = (ii < nbc && off < W) ? band[(k0 + ii) * W + off] : 0.0;
  }
#pragma unroll
  for (int jj = 0; jj < NB; ++jj)
#pragma unroll
    for (int ii = jj + 1; ii < NB; ++ii) u[ii] -= L[ii][jj] * u[jj];
#pragma unroll
  for (int ii = 0; ii < NB; ++ii) {
    const int64_t off = c - (k0 + ii) + kl;
    if (ii < nbc && off < W) band[(k0 + ii) * W + off] = u[ii];
  }
}

// A22 -= L21 U12 over rows k1 .. k1 + nrows - 1 and columns k1 .. k1 + ncols - 1
template <int NB>
__global__ void __launch_bounds__(256) k_band_update(double *band, int64_t n, int kl, int W, int64_t k0, int nrows,
                                                    int ncols, const double *__restrict__ Lbuf) {
  __shared__ double Lt[64][NB + 1];
  __shared__ double Ut[NB][64];
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
  for (int idx = threadIdx.x; idx < 64 * NB; idx += blockDim.x) {
    const int i = idx / NB, jj = idx % NB;
    const int64_t rl = (k1 - k0) + r0 + i;  // row in the panel buffer
    Lt[i][jj] = (r0 + i < nrows && jj < nbc) ? Lbuf[rl * NB + jj] : 0.0;
  }
  for (int idx = threadIdx.x; idx < 64 * NB; idx += blockDim.x) {
    const int jj = idx / 64, t = idx % 64;
    const int64_t c = k1 + c0 + t;
    const int64_t off = c - (k0 + jj) + kl;
    Ut[jj][t] = (c0 + t < ncols && jj < nbc && off < W) ? band[(k0 + jj) * W + off] : 0.0;
  }
  __syncthreads();
  const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
  double acc[4][4] = {};
#pragma unroll
  for (int jj = 0; jj < NB; ++jj) {
    double a[4], bb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = Lt[ti * 4 + u][jj];
      bb[u] = Ut[jj][tj * 4 + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * bb[v];
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = r0 + ti * 4 + u;
    if (i >= nrows) continue;
    const int64_t r = k1 + i;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int t = c0 + tj * 4 + v;
      if (t >= ncols) continue;
      const int64_t off = (k1 + t) - r + kl;
      if (off >= 0 && off < W) band[r * W + off] -= acc[u][v];
    }
  }
}

// U x = y, 32 rows at a time from the bottom
__global__ void __launch_bounds__(1024) k_band_back(const double *__restrict__ band, int64_t n, int kl, int ku,
                                                   int W, const double *__restrict__ y, double *x) {
  __shared__ double acc[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t j1 = n; j1 > 0; j1 -= 32) {
    const int64_t j0 = j1 - 32 > 0 ? j1 - 32 : 0;
    const int nr = (int)(j1 - j0);
    if (warp < nr) {
      const int64_t i = j0 + warp;
      const int64_t cend = min(n - 1, i + kl + ku);
      double s = 0.0;
      for (int64_t c = j1 + lane; c <= cend; c += 32) s += band[i * W + (c - i + kl)] * x[c];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) acc[warp] = y[i] - s;
    }
    __syncthreads();
    if (warp == 0) {
      double a = lane < nr ? acc[lane] : 0.0;
      const int64_t i = j0 + lane;
      for (int t = nr - 1; t >= 0; --t) {
        double xt = 0.0;
        if (lane == t) {
          xt = a / band[i * W + kl];
          x[i] = xt;
        }
        xt = __shfl_sync(0xffffffffu, xt, t);
        if (lane < t) {
          const int64_t off = (j0 + t) - i + kl;
          if (off < W) a -= band[i * W + off] * xt;
        }
      }
    }
    __syncthreads();
  }
}

int ensure_lu(mic_ctx *ctx, size_t need) {
  if (ctx->lu_bytes >= need) return MIC_OK;
  cudaFree(ctx->lu_buf);
  ctx->lu_buf = nullptr;
  ctx->lu_bytes = 0;
  if (cudaMalloc(&ctx->lu_buf, need) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->lu_bytes = need;
  return MIC_OK;
}

template <int NB>
int factor_solve(mic_ctx *ctx, double *band, int64_t n, int kl, int ku, int W, int *piv, double *b, int *info,
                 double *Lbuf) {
  const size_t smem = sizeof(double) * (size_t)(NB + kl) * NB;
  MIC_CUDA_TRY(cudaFuncSetAttribute(k_band_panel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for (int64_t k0 = 0; k0 < n; k0 += NB) {
    const int64_t k1 = std::min<int64_t>(k0 + NB, n);
    {
      MIC_KERNEL(ctx, "k_band_panel");
      k_band_panel<NB><<<1, kPanelThreads, smem, ctx->stream>>>(band, n, kl, ku, W, k0, piv, b, info, Lbuf);
    }
    if (k1 >= n) break;
    const int ncols = (int)(std::min<int64_t>(n - 1, k1 - 1 + kl + ku) - k1 + 1);
    const int nrows = (int)(std::min<int64_t>(n - 1, k1 - 1 + kl) - k1 + 1);
    if (ncols > 0) {
      MIC_KERNEL(ctx, "k_band_trsm");
      k_band_trsm<NB><<<(ncols + 127) / 128, 128, 0, ctx->stream>>>(band, n, kl, W, k0, ncols, Lbuf);
    }
    if (ncols > 0 && nrows > 0) {
      MIC_KERNEL(ctx, "k_band_update");
      dim3 g((ncols + 63) / 64, (nrows + 63) / 64);
      k_band_update<NB><<<g, 256, 0, ctx->stream>>>(band, n, kl, W, k0, nrows, ncols, Lbuf);
    }
  }
  return MIC_OK;
}

template <typename T>
T *carve(unsigned char *&p, size_t count) {
  T *r = reinterpret_cast<T *>(p);
  p += ((count * sizeof(T) + 255) / 256) * 256;
  return r;
}

}  // namespace

extern "C" int mic_linear_solve(mic_ctx *ctx, int which) {
  if (!ctx || which < 0 || which > 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  mic_system_store &S = ctx->sys[which];
  if (!S.cnt) return MIC_ERR_ARG;
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const int dof = which == 0 ? 3 : 1;
  const int64_t n = S.n;
  const int transpose = NX > NY ? 1 : 0;
  // band widths under the ordering
  int *bw = nullptr;
  {
    int e = ensure_lu(ctx, 4096);
    if (e) return e;
    bw = static_cast<int *>(ctx->lu_buf);
    MIC_CUDA_TRY(cudaMemsetAsync(bw, 0, 2 * sizeof(int), ctx->stream));
    MIC_KERNEL(ctx, "k_band_width");
    k_band_width<<<grid_for(n), kBlock, 0, ctx->stream>>>(S.cnt, S.col, S.width, n, dof, NX, NY, transpose, bw);
  }
  int hbw[2];
  MIC_CUDA_TRY(cudaMemcpyAsync(hbw, bw, sizeof(hbw), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const int kl = hbw[0], ku = hbw[1];
  const int W = 2 * kl + ku + 1;
  const size_t kSmemMax = 200 * 1024;
  int nb = 0;
  for (int cand : {32, 16, 8})
    if (sizeof(double) * (size_t)(cand + kl) * cand <= kSmemMax) {
      nb = cand;
      break;
    }
  if (!nb) return MIC_ERR_SOLVE;  // band wider than a panel in shared memory
  const size_t lbuf = (size_t)(nb + kl) * nb;
  const size_t need = 256 + (((size_t)n * W * sizeof(double) + 255) / 256) * 256 +
                      3 * (((size_t)n * 8 + 255) / 256) * 256 + ((lbuf * 8 + 255) / 256) * 256 + 256;
  int e = ensure_lu(ctx, need);
  if (e) return e;
  unsigned char *p = static_cast<unsigned char *>(ctx->lu_buf);
  int *info = carve<int>(p, 64);
  double *band = carve<double>(p, (size_t)n * W);
  double *b = carve<double>(p, n);
  double *x = carve<double>(p, n);
  int *piv = carve<int>(p, n);
  double *Lbuf = carve<double>(p, lbuf);
  MIC_CUDA_TRY(cudaMemsetAsync(band, 0, sizeof(double) * (size_t)n * W, ctx->stream));
  const int big = INT_MAX;
  MIC_CUDA_TRY(cudaMemcpyAsync(info, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  {
    MIC_KERNEL(ctx, "k_band_scatter");
    k_band_scatter<<<grid_for(n), kBlock, 0, ctx->stream>>>(S.cnt, S.col, S.val, S.rhs, S.width, n, dof, NX, NY,
                                                            transpose, kl, W, band, b);
  }
  if (nb == 32)
    e = factor_solve<32>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf);
  else if (nb == 16)
    e = factor_solve<16>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf);
  else
    e = factor_solve<8>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf);
  if (e) return e;
  {
    MIC_KERNEL(ctx, "k_band_back");
    k_band_back<<<1, 1024, 0, ctx->stream>>>(band, n, kl, ku, W, b, x);
  }
  double *out = nullptr;
  if (which == 0) {
    if (!ctx->solution && cudaMalloc((void **)&ctx->solution, sizeof(double) * n) != cudaSuccess) return MIC_ERR_NOMEM;
    out = ctx->solution;
  } else {
    out = ctx->nodal[MIC_NF_THIST];
  }
  {
    MIC_KERNEL(ctx, "k_band_gather");
    k_band_gather<<<grid_for(n), kBlock, 0, ctx->stream>>>(x, n, dof, NX, NY, transpose, out);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  int hinfo = 0;
  MIC_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  S.factored = 1;
  S.kl = kl;
  S.ku = ku;
  S.zero_pivot = hinfo == INT_MAX ? -1 : hinfo;
  return hinfo == INT_MAX ? MIC_OK : MIC_ERR_SOLVE;
}

extern "C" int mic_solution_get(mic_ctx *ctx, int which, double *out) {
  if (!ctx || !out || which < 0 || which > 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  const double *src = which == 0 ? ctx->solution : ctx->nodal[MIC_NF_THIST];
  if (!src) return MIC_ERR_ARG;
  MIC_CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * (which == 0 ? 3 * nn : nn), cudaMemcpyDeviceToHost,
                               ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_system_band(mic_ctx *ctx, int which, int *kl, int *ku) {
  if (!ctx || which < 0 || which > 1) return MIC_ERR_ARG;
  if (kl) *kl = ctx->sys[which].kl;
  if (ku) *ku = ctx->sys[which].ku;
  return MIC_OK;
}
