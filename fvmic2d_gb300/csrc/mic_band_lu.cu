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
// Factorisation, right-looking in panels of NB columns (16, or 8 when the window of NB + kl rows
// would not fit one CTA at one row per thread):
//   panel  one CTA, each window row in one thread's registers, column by column: pivot row
//          (largest |value|, first on ties), interchange (whole panel rows, the right-hand side
//          too), multipliers, rank-1 update of the panel; the forward substitution of the
//          right-hand side rides along (it is one more column);
//   trsm   the trailing columns of the rows whose position changed follow them (a gather), then
//          U12 = L11^-1 A12 for the columns right of the panel, a warp per column;
//   update A22 -= L21 U12 over the band window, 32 x 32 tiles: the next panel's columns on the
//          main stream, the rest on a side stream, overlapping the next panel.
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

// One panel: columns k0 .. k1-1 and the window rows k0 .. k0+R-1 (R <= 1024).  Thread r holds
// window row r in registers (its NB panel columns and its right-hand side entry), fully unrolled
// over the panel's columns, so a column step is: the pivot search over the column (integer images
// of |a|: ordered for non-negative doubles, NaN skipped, off the FP64 pipe), the pivot row and
// the row it displaces published in shared memory, one reciprocal, and every row below forming
// its multiplier and updating itself against the broadcast pivot row.  Interchanges move whole
// panel rows (multipliers included, so that L ends in final row order for the deferred trsm and
// update) and the right-hand side; the trailing columns of the rows whose position changed
// follow in the trsm (the list of moved rows goes to `moved`).
template <int NB, int MAXT>
__global__ void __launch_bounds__(MAXT) k_band_panel(double *band, int64_t n, int kl, int ku, int W, int64_t k0,
                                                    int *piv, double *b, int *info, double *Lbuf, int *moved) {
  __shared__ double sA[NB + 1];  // the pivot row (new row jj) and its right-hand side
  __shared__ double sB[NB + 1];  // row jj, which moves to the pivot's position
  __shared__ long long red_v[MAXT / 32];
  __shared__ int red_i[MAXT / 32];
  __shared__ int who[MAXT];      // the window row now at each position
  __shared__ int s_piv[NB];
  __shared__ double s_rcp;
  __shared__ int s_nchg;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  const int R = (int)(min(n, k1 + kl) - k0);
  const bool own = tid < R;
  double row[NB];
  double brow = 0.0;
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    const int off = c - tid + kl;
    row[c] = (own && c < nbc && off >= 0 && off < W) ? band[(k0 + tid) * (int64_t)W + off] : 0.0;
  }
  if (own) {
    brow = b[k0 + tid];
    who[tid] = tid;
  }
  __syncthreads();
#pragma unroll
  for (int jj = 0; jj < NB; ++jj) {
    if (jj >= nbc) break;
    const int rmax = (int)(min(n - 1, k0 + jj + kl) - k0);
    // pivot: largest |a|, the first of equal ones (LAPACK's idamax)
    long long bv = -1;
    int bi = INT_MAX;
    if (own && tid >= jj && tid <= rmax) {
      const long long a = dbits(row[jj]) & 0x7fffffffffffffffLL;
      if (a <= 0x7ff0000000000000LL) {
        bv = a;
        bi = tid;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const long long v2 = __shfl_down_sync(0xffffffffu, bv, o);
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
    bv = red_v[0];
    bi = red_i[0];
    for (int w = 1; w < nwarps; ++w)
      if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bi)) {
        bv = red_v[w];
        bi = red_i[w];
      }
    const int p = (bi >= jj && bi <= rmax) ? bi : jj;  // all NaN: keep the diagonal
    if (tid == p) {
#pragma unroll
      for (int c = 0; c < NB; ++c) sA[c] = row[c];
      sA[NB] = brow;
      s_rcp = row[jj] != 0.0 ? 1.0 / row[jj] : 0.0;  // the column's one division
    }
    if (tid == jj && p != jj) {
#pragma unroll
      for (int c = 0; c < NB; ++c) sB[c] = row[c];
      sB[NB] = brow;
    }
    if (tid == 0) {
      s_piv[jj] = p;
      const int w2 = who[jj];
      who[jj] = who[p];
      who[p] = w2;
    }
    __syncthreads();
    const double rcp = s_rcp;
    if (tid == jj) {
#pragma unroll
      for (int c = 0; c < NB; ++c) row[c] = sA[c];
      brow = sA[NB];
    } else if (tid == p) {
#pragma unroll
      for (int c = 0; c < NB; ++c) row[c] = sB[c];
      brow = sB[NB];
    }
    if (rcp == 0.0) {
      if (tid == 0) atomicMin(info, (int)(k0 + jj));
      continue;
    }
    if (own && tid > jj && tid <= rmax) {
      const double l = row[jj] * rcp;  // LAPACK's scaling by the pivot's reciprocal
      row[jj] = l;
#pragma unroll
      for (int c = jj + 1; c < NB; ++c) row[c] -= l * sA[c];
      brow -= l * sA[NB];
    }
  }
  // U of the panel rows back into the band; the whole panel (L11 and L21, which interchanges can
  // carry outside the band) to the dense panel buffer; the right-hand side; the pivots
  if (own) {
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const int off = c - tid + kl;
      if (c < nbc && c >= tid && off < W) band[(k0 + tid) * (int64_t)W + off] = row[c];
      Lbuf[(int64_t)tid * NB + c] = row[c];
    }
    b[k0 + tid] = brow;
  }
  __syncthreads();
  for (int jj = tid; jj < nbc; jj += blockDim.x) piv[k0 + jj] = (int)(k0 + s_piv[jj]);
  // the positions whose row changed and the window row each now holds, for the trsm's gather
  if (tid == 0) s_nchg = 0;
  __syncthreads();
  if (own && who[tid] != tid) {
    const int q = atomicAdd(&s_nchg, 1);
    moved[1 + 2 * q] = tid;
    moved[2 + 2 * q] = who[tid];
  }
  __syncthreads();
  if (tid == 0) moved[0] = s_nchg;
}

// U12 = L11^-1 A12: columns k1 .. k1 + ncols - 1, a warp per column (lane ii holds row ii), so the
// columns spread over all SMs.  First the column's entries of the rows the panel moved follow
// them: every nonzero an interchange at step j moves lies in columns j .. j + kl + ku, inside this
// range, so the gather is complete here; each warp reads all the moved entries of its column
// before it writes any.
template <int NB>
__global__ void __launch_bounds__(256) k_band_trsm(double *band, int64_t n, int kl, int ku, int W, int64_t k0,
                                                  int ncols, const double *__restrict__ Lbuf,
                                                  const int *__restrict__ moved) {
  __shared__ double L[NB][NB + 1];
  __shared__ int mv[4 * NB + 1];
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int ii = idx / NB, jj = idx % NB;
    L[ii][jj] = (ii > jj && ii < nbc) ? Lbuf[idx] : 0.0;
  }
  const int nm = moved[0];  // at most 2 NB rows change position
  for (int idx = threadIdx.x; idx < 2 * nm; idx += blockDim.x) mv[idx] = moved[1 + idx];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= ncols) return;
  const int64_t c = k1 + t;
  constexpr int PERM = (2 * NB + 31) / 32;
  double v[PERM];
#pragma unroll
  for (int q = 0; q < PERM; ++q) {
    const int e = lane + 32 * q;
    v[q] = 0.0;
    if (e < nm) {
      const int64_t go = k0 + mv[2 * e + 1];
      if (c <= go + kl + ku) v[q] = band[go * W + (c - go + kl)];
    }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < PERM; ++q) {
    const int e = lane + 32 * q;
    if (e < nm) {
      const int64_t gi = k0 + mv[2 * e];
      if (c <= gi + kl + ku) band[gi * W + (c - gi + kl)] = v[q];
    }
  }
  __syncwarp();
  const int64_t off = c - (k0 + lane) + kl;
  const bool mine = lane < nbc && off < W;
  double u = mine ? band[(k0 + lane) * W + off] : 0.0;
#pragma unroll
  for (int jj = 0; jj < NB; ++jj) {
    const double uj = __shfl_sync(0xffffffffu, u, jj);
    if (lane > jj && lane < NB) u -= L[lane < NB ? lane : 0][jj] * uj;
  }
  if (mine) band[(k0 + lane) * W + off] = u;
}

// A22 -= L21 U12 over rows k1 .. k1 + nrows - 1 and columns k1 + coff .. k1 + coff + ncols - 1,
// 32 x 32 tiles
// (the FP64 pipe is the bound: small tiles spread one panel's update over all SMs)
constexpr int kTile = 32;
template <int NB>
__global__ void __launch_bounds__(256) k_band_update(double *band, int64_t n, int kl, int W, int64_t k0, int nrows,
                                                    int coff, int ncols, const double *__restrict__ Lbuf) {
  __shared__ double Lt[kTile][NB + 1];
  __shared__ double Ut[NB][kTile + 1];
  const int64_t k1 = min(k0 + NB, n);
  const int nbc = (int)(k1 - k0);
  const int r0 = blockIdx.y * kTile, c0 = blockIdx.x * kTile;
  for (int idx = threadIdx.x; idx < kTile * NB; idx += blockDim.x) {
    const int i = idx / NB, jj = idx % NB;
    const int64_t rl = nbc + r0 + i;  // row in the panel buffer
    Lt[i][jj] = (r0 + i < nrows && jj < nbc) ? Lbuf[rl * NB + jj] : 0.0;
  }
  for (int idx = threadIdx.x; idx < kTile * NB; idx += blockDim.x) {
    const int jj = idx / kTile, t = idx % kTile;
    const int64_t c = k1 + coff + c0 + t;
    const int64_t off = c - (k0 + jj) + kl;
    Ut[jj][t] = (c0 + t < ncols && jj < nbc && off < W) ? band[(k0 + jj) * W + off] : 0.0;
  }
  __syncthreads();
  const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;  // rows ti, ti+16; columns tj, tj+16
  double acc[2][2] = {};
#pragma unroll 8
  for (int jj = 0; jj < NB; ++jj) {
    const double a0 = Lt[ti][jj], a1 = Lt[ti + 16][jj];
    const double b0 = Ut[jj][tj], b1 = Ut[jj][tj + 16];
    acc[0][0] += a0 * b0;
    acc[0][1] += a0 * b1;
    acc[1][0] += a1 * b0;
    acc[1][1] += a1 * b1;
  }
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int i = r0 + ti + 16 * u;
    if (i >= nrows) continue;
    const int64_t r = k1 + i;
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int t = c0 + tj + 16 * v;
      if (t >= ncols) continue;
      const int64_t off = (k1 + coff + t) - r + kl;
      if (off >= 0 && off < W) band[r * W + off] -= acc[u][v];
    }
  }
}

// U x = y, 32 rows at a time from the bottom: a warp per row for the part from solved unknowns,
// the 32 x 32 diagonal block staged in shared memory, one warp for the triangle
__global__ void __launch_bounds__(1024) k_band_back(const double *__restrict__ band, int64_t n, int kl, int ku,
                                                   int W, const double *__restrict__ y, double *x) {
  __shared__ double acc[32];
  __shared__ double Ud[32][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t j1 = n; j1 > 0; j1 -= 32) {
    const int64_t j0 = j1 - 32 > 0 ? j1 - 32 : 0;
    const int nr = (int)(j1 - j0);
    if (warp < nr) {
      const int64_t i = j0 + warp;
      const int64_t cend = min(n - 1, i + kl + ku);
      double s = 0.0;
#pragma unroll 4
      for (int64_t c = j1 + lane; c <= cend; c += 32) s += band[i * W + (c - i + kl)] * x[c];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) acc[warp] = y[i] - s;
      const int64_t off = (j0 + lane) - i + kl;  // row `warp` of the diagonal block, column `lane`
      Ud[warp][lane] = (lane >= warp && lane < nr && off < W) ? band[i * W + off] : 0.0;
    }
    __syncthreads();
    if (warp == 0) {
      double a = lane < nr ? acc[lane] : 0.0;
      const double rd = 1.0 / (lane < nr ? Ud[lane][lane] : 1.0);  // all lanes' divisions at once
      for (int t = nr - 1; t >= 0; --t) {
        double xt = 0.0;
        if (lane == t) xt = a * rd;
        xt = __shfl_sync(0xffffffffu, xt, t);
        if (lane < t) a -= Ud[lane][t] * xt;
        if (lane == t) a = xt;
      }
      if (lane < nr) x[j0 + lane] = a;
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

// The update of panel k splits in two: its first NB columns (the next panel's) on the main
// stream, the rest on the side stream, where it runs while panel k+1 factors (the panel touches
// only its own columns; the trailing columns of its interchanged rows move in its trsm, which
// waits for the side stream).  The dense panel buffer alternates between two halves, so that
// panel k+1 does not overwrite the L21 the side stream is still reading.
template <int NB, int MAXT>
int factor_solve(mic_ctx *ctx, double *band, int64_t n, int kl, int ku, int W, int *piv, double *b, int *info,
                 double *Lbuf2, size_t lhalf, int *moved) {
  cudaStream_t side = ctx->lu_side;
  cudaEvent_t ev_trsm = ctx->lu_ev[0], ev_far = ctx->lu_ev[1];
  bool far_pending = false;
  int parity = 0;
  for (int64_t k0 = 0; k0 < n; k0 += NB, parity ^= 1) {
    const int64_t k1 = std::min<int64_t>(k0 + NB, n);
    const int R = (int)(std::min<int64_t>(n, k1 + kl) - k0);
    double *Lbuf = Lbuf2 + parity * lhalf;
    {
      MIC_KERNEL(ctx, "k_band_panel");
      k_band_panel<NB, MAXT><<<1, (R + 31) / 32 * 32, 0, ctx->stream>>>(band, n, kl, ku, W, k0, piv, b, info, Lbuf,
                                                                        moved);
    }
    if (k1 >= n) break;
    const int ncols = (int)(std::min<int64_t>(n - 1, k1 - 1 + kl + ku) - k1 + 1);
    const int nrows = (int)(std::min<int64_t>(n - 1, k1 - 1 + kl) - k1 + 1);
    if (far_pending) MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_far, 0));
    far_pending = false;
    if (ncols > 0) {
      MIC_KERNEL(ctx, "k_band_trsm");
      k_band_trsm<NB><<<(ncols + 7) / 8, 256, 0, ctx->stream>>>(band, n, kl, ku, W, k0, ncols, Lbuf, moved);
    }
    if (ncols > 0 && nrows > 0) {
      const int nnear = std::min(NB, ncols), nfar = ncols - nnear;
      if (nfar > 0) MIC_CUDA_TRY(cudaEventRecord(ev_trsm, ctx->stream));
      {
        MIC_KERNEL(ctx, "k_band_update");
        dim3 g((nnear + kTile - 1) / kTile, (nrows + kTile - 1) / kTile);
        k_band_update<NB><<<g, 256, 0, ctx->stream>>>(band, n, kl, W, k0, nrows, 0, nnear, Lbuf);
      }
      if (nfar > 0) {
        MIC_CUDA_TRY(cudaStreamWaitEvent(side, ev_trsm, 0));
        dim3 g((nfar + kTile - 1) / kTile, (nrows + kTile - 1) / kTile);
        k_band_update<NB><<<g, 256, 0, side>>>(band, n, kl, W, k0, nrows, nnear, nfar, Lbuf);
        ++ctx->launches;
        MIC_CUDA_TRY(cudaEventRecord(ev_far, side));
        far_pending = true;
      }
    }
  }
  if (far_pending) MIC_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_far, 0));
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
  // panel width: the window's NB + kl rows are one thread each (at most 1024).  16 columns: 32
  // halved the panel's launches but doubled its unrolled code and its per-column FP64 work, and
  // was slower at every size measured (band 65 to 392)
  int nb = 0;
  if (16 + kl <= 1024)
    nb = 16;
  else if (8 + kl <= 1024)
    nb = 8;
  if (!nb) return MIC_ERR_SOLVE;  // band wider than one panel window
  const size_t lbuf = (((size_t)(nb + kl) * nb + 31) / 32) * 32;  // one half of the panel buffer
  const size_t mbuf = 1 + 4 * 32;  // count, then (position, window row) pairs, at most 2 NB
  const size_t need = 256 + (((size_t)n * W * sizeof(double) + 255) / 256) * 256 +
                      3 * (((size_t)n * 8 + 255) / 256) * 256 + ((2 * lbuf * 8 + 255) / 256) * 256 +
                      ((mbuf * 4 + 255) / 256) * 256 + 256;
  int e = ensure_lu(ctx, need);
  if (e) return e;
  if (!ctx->lu_side) {
    MIC_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->lu_side, cudaStreamNonBlocking));
    MIC_CUDA_TRY(cudaEventCreateWithFlags(&ctx->lu_ev[0], cudaEventDisableTiming));
    MIC_CUDA_TRY(cudaEventCreateWithFlags(&ctx->lu_ev[1], cudaEventDisableTiming));
  }
  unsigned char *p = static_cast<unsigned char *>(ctx->lu_buf);
  int *info = carve<int>(p, 64);
  double *band = carve<double>(p, (size_t)n * W);
  double *b = carve<double>(p, n);
  double *x = carve<double>(p, n);
  int *piv = carve<int>(p, n);
  double *Lbuf = carve<double>(p, 2 * lbuf);
  int *moved = carve<int>(p, mbuf);
  MIC_CUDA_TRY(cudaMemsetAsync(band, 0, sizeof(double) * (size_t)n * W, ctx->stream));
  const int big = INT_MAX;
  MIC_CUDA_TRY(cudaMemcpyAsync(info, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  {
    MIC_KERNEL(ctx, "k_band_scatter");
    k_band_scatter<<<grid_for(n), kBlock, 0, ctx->stream>>>(S.cnt, S.col, S.val, S.rhs, S.width, n, dof, NX, NY,
                                                            transpose, kl, W, band, b);
  }
  auto factor = [&]() -> int {
    if (nb == 32) return factor_solve<32, 512>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf, lbuf, moved);
    if (nb == 16) return factor_solve<16, 1024>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf, lbuf, moved);
    return factor_solve<8, 1024>(ctx, band, n, kl, ku, W, piv, b, info, Lbuf, lbuf, moved);
  };
  // The factorisation is 3-4 launches and two stream hand-offs per panel, the same sequence for
  // every solve of a system of this shape (the band comes from the grid's stencil): captured once
  // as a graph and replayed, so host launch cost stops gating the panels.  Not while launches are
  // being timed one by one, and not beyond 20,000 panels (instantiation cost).
  const bool graphable = !ctx->prof_on && (n + nb - 1) / nb <= 20000;
  if (graphable && S.lu_exec && S.lu_key_buf == ctx->lu_buf && S.lu_key_n == n && S.lu_key_kl == kl &&
      S.lu_key_ku == ku && S.lu_key_nb == nb) {
    MIC_CUDA_TRY(cudaGraphLaunch(S.lu_exec, ctx->stream));
    ctx->launches += S.lu_nodes;
  } else if (graphable && cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
    const long long l0 = ctx->launches;
    e = factor();
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (e || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return e ? e : mic_fail_cuda(ctx, ce);
    }
    if (S.lu_exec) cudaGraphExecDestroy(S.lu_exec);
    S.lu_exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&S.lu_exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      S.lu_exec = nullptr;
      return mic_fail_cuda(ctx, ie);
    }
    S.lu_nodes = ctx->launches - l0;
    S.lu_key_buf = ctx->lu_buf;
    S.lu_key_n = n;
    S.lu_key_kl = kl;
    S.lu_key_ku = ku;
    S.lu_key_nb = nb;
    MIC_CUDA_TRY(cudaGraphLaunch(S.lu_exec, ctx->stream));
  } else {
    cudaGetLastError();  // a stream that cannot be captured: launch directly
    e = factor();
    if (e) return e;
  }
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
