// mic_bin_sort.cu -- K1: cell location (findMarkerCells, markers.c:41-106) and the stable
// counting sort that orders the device marker columns by cell.
//
// Cell location uses integer compares on the IEEE bit patterns of X, Y and the gridlines
// (valid because every compared value is non-negative): the same answer as the reference's
// bisection, with no FP64 instructions on a GPU whose FP64 rate is 1/60 of FP32.
//
// Sorting: key = 4*(cellY*NCX + cellX) + 2*qy + qx, where (qx, qy) is the marker's quadrant of
// its cell (X >= xc[cellX+1], Y >= yc[cellY+1]: the stagger test of findCellStag2D) and NCX the
// basic cells in x (NX - 1, or NX on a grid periodic in x: markers.c:49, 73); out-of-domain
// markers get key 4*NCX*(NY-1).  Cells stay contiguous and inside a cell the markers
// of each quadrant are contiguous, so every staggered (cell-centre) cell's markers are four
// runs.  An LSD radix sort with 8-bit digits (stable by construction) orders (key, index) pairs:
// per 4096-marker tile a digit histogram, one exclusive scan over the digit-major
// histogram matrix, then a scatter in which each tile ranks its items per digit with warp
// match/ballot in index order.  Ties keep the current device order, so the result equals
// a CPU stable sort of the current order.  cell_start[] brackets each cell's markers.
#include "mic_internal.cuh"

using namespace mic;

namespace {

constexpr int kSortThreads = 256;
constexpr int kItemsPerThread = 16;
constexpr int kTile = kSortThreads * kItemsPerThread;  // 4096
constexpr int kRadixBits = 8;
constexpr int kBuckets = 1 << kRadixBits;

// Largest i in [0, n-2] with g[i] <= v (markers.c:47-69), on bit patterns.
__device__ __forceinline__ int bisect_bits(const long long *__restrict__ g, int n, long long v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (v >= __ldg(g + mid))
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// The same index from a hint, the marker's cell before this binning: most markers stay in it or
// move to a neighbour, whose intervals g[h] <= v < g[h+1] (the last index takes every v >= g[n-2])
// are tested first; otherwise, or for a hint out of [0, n-2], the bisection.  The tested interval
// characterises the largest i with g[i] <= v, so the result is the bisection's for any hint.
__device__ __forceinline__ int locate_bits(const long long *__restrict__ g, int n, long long v, int hint) {
  if (hint >= 0 && hint <= n - 2) {
    if (__ldg(g + hint) <= v) {
      if (hint == n - 2 || v < __ldg(g + hint + 1)) return hint;
      // v >= g[hint + 1]
      if (hint + 1 == n - 2 || v < __ldg(g + hint + 2)) return hint + 1;
    } else if (hint >= 1 && __ldg(g + hint - 1) <= v) {
      return hint - 1;  // g[hint - 1] <= v < g[hint]
    }
  }
  return bisect_bits(g, n, v);
}

__global__ void k_find_cells(Params P, const double *__restrict__ X, const double *__restrict__ Y,
                             int *__restrict__ cellX, int *__restrict__ cellY, int *__restrict__ cpu,
                             int *__restrict__ key, int64_t n, Status *st) {
  __shared__ unsigned long long s_out;
  if (threadIdx.x == 0) s_out = 0;
  __syncthreads();
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < n) {
    const long long bx = dbits(X[m]);
    const long long by = dbits(Y[m]);
    const long long ux = (bx == (long long)0x8000000000000000ULL) ? 0LL : bx;
    const long long uy = (by == (long long)0x8000000000000000ULL) ? 0LL : by;
    const long long blx = dbits(P.LX), bly = dbits(P.LY);
    // X >= 0 && Y >= 0 && X <= LX && Y <= LY; NaN fails every test
    const bool in = ux >= 0 && uy >= 0 && ux <= blx && uy <= bly;
    const int hx = cellX[m], hy = cellY[m];  // the cell before this binning (any value)
    int cx = -1, cy = -1, k = 4 * P.NCX * (P.NY - 1);
    if (in) {
      cx = locate_bits(P.xbits, P.NCX + 1, ux, hx);  // lines 0..NCX (periodic: line NX = LX)
      cy = locate_bits(P.ybits, P.NY, uy, hy);
      const int qx = ux >= nonneg_bits(P.xc[cx + 1]), qy = uy >= nonneg_bits(P.yc[cy + 1]);
      k = 4 * (cy * P.NCX + cx) + 2 * qy + qx;
    } else {
      atomicAdd(&s_out, 1ULL);
    }
    cellX[m] = cx;
    cellY[m] = cy;
    cpu[m] = 0;
    key[m] = k;
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_out) atomicAdd(&st->n_out, s_out);
}

__global__ void k_radix_hist(const int *__restrict__ key, int64_t n, int shift, int *__restrict__ hist,
                             int ntiles) {
  __shared__ int cnt[kBuckets];
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll 4
  for (int r = 0; r < kItemsPerThread; ++r) {
    const int64_t idx = base + (int64_t)r * kSortThreads + threadIdx.x;
    if (idx < n) atomicAdd(&cnt[(key[idx] >> shift) & (kBuckets - 1)], 1);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) hist[(size_t)b * ntiles + blockIdx.x] = cnt[b];
}

// In-place exclusive scan of an int array of length len, in blocks of 2048; block totals go
// to aux[] and are scanned by the same routine recursively from the host.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanBlock = kScanThreads * kScanPer;

__global__ void k_scan_block(int *__restrict__ data, int64_t len, int *__restrict__ block_sums) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
  int v[kScanPer];
  int sum = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = (base + k < len) ? data[base + k] : 0;
    sum += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = wi - w;
    if (lane == kScanThreads / 32 - 1 && block_sums) block_sums[blockIdx.x] = wi;
  }
  __syncthreads();
  int run = warp_tot[warp] + incl - sum;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < len) data[base + k] = run;
    run += v[k];
  }
}

__global__ void k_scan_add(int *__restrict__ data, int64_t len, const int *__restrict__ block_offsets) {
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  const int add = block_offsets[blockIdx.x];
  for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x)
    if (base + k < len) data[base + k] += add;
}

__global__ void k_radix_scatter(const int *__restrict__ key_in, const int *__restrict__ val_in, int use_iota,
                                int *__restrict__ key_out, int *__restrict__ val_out, int64_t n, int shift,
                                const int *__restrict__ hist, int ntiles) {
  __shared__ int tile_off[kBuckets];
  __shared__ int run[kBuckets];
  __shared__ int wcnt[kSortThreads / 32][kBuckets];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) {
    tile_off[b] = hist[(size_t)b * ntiles + blockIdx.x];
    run[b] = 0;
  }
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int r = 0; r < kItemsPerThread; ++r) {
    for (int t = threadIdx.x; t < (kSortThreads / 32) * kBuckets; t += blockDim.x) (&wcnt[0][0])[t] = 0;
    __syncthreads();
    const int64_t idx = base + (int64_t)r * kSortThreads + threadIdx.x;
    const bool valid = idx < n;
    int k = 0, v = 0, d = kBuckets;  // invalid items form their own group and are never written
    if (valid) {
      k = key_in[idx];
      v = use_iota ? (int)idx : val_in[idx];
      d = (k >> shift) & (kBuckets - 1);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt_mask);
    if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    // per digit: exclusive prefix over the warps of this round, then advance the running count
    for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) {
      int acc = run[b];
#pragma unroll
      for (int w = 0; w < kSortThreads / 32; ++w) {
        int c = wcnt[w][b];
        wcnt[w][b] = acc;
        acc += c;
      }
      run[b] = acc;
    }
    __syncthreads();
    if (valid) {
      const int pos = tile_off[d] + wcnt[warp][d] + rank;
      key_out[pos] = k;
      val_out[pos] = v;
    }
    __syncthreads();
  }
}

// From the sorted (cell, quadrant) keys: qs[q] = first sorted position with key >= q for
// q in [0, 4*ncells+4] (when qs is given) and cs[c] = qs[4c] for c in [0, ncells+1].
__global__ void k_cell_start(const int *__restrict__ skey, int64_t n, int ncells, int *__restrict__ cs,
                             int *__restrict__ qs) {
  // one thread per (cell, quadrant) key q in [0, 4 ncells + 4]: the run of key q starts at the
  // first sorted position whose key is >= q (n when there is none), so empty stretches of cells
  // cost nothing extra.  cs[c] = qs[4c].  The search starts at the position q would have with
  // markers spread evenly over the keys and gallops outwards (steps 1, 2, 4, ...) until it
  // brackets the answer, then bisects the bracket: a few loads, near those of the neighbouring
  // threads, where a bisection of the whole array takes log2 n.  Invariant of the final
  // bisection: every position below lo holds a key < q, and hi is n or holds a key >= q.
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t qmax = 4LL * ncells + 4;
  if (q > qmax) return;
  int64_t lo = 0, hi = n;
  if (n > 0) {
    const int64_t g = q * n / (qmax + 1);  // in [0, n)
    if (skey[g] < q) {
      lo = g + 1;
      for (int64_t step = 1;; step <<= 1) {
        const int64_t p = g + step;
        if (p >= n) break;  // hi stays n
        if (skey[p] >= q) {
          hi = p;
          break;
        }
        lo = p + 1;
      }
    } else {
      hi = g;
      for (int64_t step = 1;; step <<= 1) {
        const int64_t p = g - step;
        if (p < 0) break;  // lo stays 0
        if (skey[p] < q) {
          lo = p + 1;
          break;
        }
        hi = p;
      }
    }
  }
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (skey[mid] < q)
      lo = mid + 1;
    else
      hi = mid;
  }
  if (qs) qs[q] = (int)lo;
  if ((q & 3) == 0) cs[q >> 2] = (int)lo;
}

struct GatherCols {
  const double *src_f[C_F64_COUNT];
  double *dst_f[C_F64_COUNT];
  const int *src_i[C_I32_COUNT];
  int *dst_i[C_I32_COUNT];
  int nf;  // double columns moved: the device-only grain column only once grain sizes were set
};

// The gather of every column into the sorted order.  GEO: also the projection geometry of each
// marker, from the position and cell just gathered: this kernel is bound by HBM and the
// geometry by the FP64 pipe, so together they cost little more than the gather alone.
// Every load comes before the first store.  The compiler cannot tell the column buffers apart,
// so a load written after a store could not issue before it: interleaved, each thread would
// wait out one memory latency per column (30 in a row) and the gather would be bound by latency.
// The geometry's grid-line loads come before the stores for the same reason.
template <bool GEO>
__global__ void k_reorder(GatherCols g, const int *__restrict__ perm, int64_t n, Params P, GeoOut go) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int p = perm[k];
  double vf[C_F64_COUNT];
  int vi[C_I32_COUNT];
#pragma unroll
  for (int c = 0; c < C_F64_COUNT; ++c) vf[c] = (c < g.nf) ? __ldg(g.src_f[c] + p) : 0.0;
#pragma unroll
  for (int c = 0; c < C_I32_COUNT; ++c) vi[c] = __ldg(g.src_i[c] + p);
  if (GEO) geometry_marker(P, vf[C_X], vf[C_Y], vi[C_CELLX], vi[C_CELLY], go, k);
#pragma unroll
  for (int c = 0; c < C_F64_COUNT; ++c)
    if (c < g.nf) g.dst_f[c][k] = vf[c];
#pragma unroll
  for (int c = 0; c < C_I32_COUNT; ++c) g.dst_i[c][k] = vi[c];
}

// perm[k] = device slot of caller marker k (k < n); slots from n on stay in place
__global__ void k_restore_perm(const int *__restrict__ id, int64_t n, int64_t cap, int *__restrict__ perm) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= cap) return;
  if (s < n)
    perm[id[s]] = (int)s;
  else
    perm[s] = (int)s;
}

// aux: free space for the block totals of this level and all coarser levels
int scan_exclusive(mic_ctx *ctx, int *data, int64_t len, int *aux) {
  const int64_t nb = (len + kScanBlock - 1) / kScanBlock;
  if (nb <= 1) {
    {
      MIC_KERNEL(ctx, "k_scan_block");
      k_scan_block<<<1, kScanThreads, 0, ctx->stream>>>(data, len, nullptr);
    }
    return cudaGetLastError() == cudaSuccess ? MIC_OK : MIC_ERR_CUDA;
  }
  int *sums = aux;
  {
    MIC_KERNEL(ctx, "k_scan_block");
    k_scan_block<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(data, len, sums);
  }
  int e = scan_exclusive(ctx, sums, nb, aux + nb + 1);
  if (e) return e;
  {
    MIC_KERNEL(ctx, "k_scan_add");
    k_scan_add<<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(data, len, sums);
  }
  return cudaGetLastError() == cudaSuccess ? MIC_OK : MIC_ERR_CUDA;
}

int ensure_sort_scratch(mic_ctx *ctx, int ntiles) {
  const int64_t need = (int64_t)kBuckets * ntiles;
  if (ctx->hist_cap >= need) return MIC_OK;
  cudaFree(ctx->hist);
  cudaFree(ctx->scan_aux);
  ctx->hist = nullptr;
  ctx->scan_aux = nullptr;
  ctx->hist_cap = 0;
  if (cudaMalloc((void **)&ctx->hist, sizeof(int) * need) != cudaSuccess) return MIC_ERR_NOMEM;
  int64_t aux = 0, l = need;
  while (l > 1) {
    l = (l + kScanBlock - 1) / kScanBlock;
    aux += l + 1;
  }
  if (cudaMalloc((void **)&ctx->scan_aux, sizeof(int) * (aux + 16)) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->hist_cap = (int)need;
  return MIC_OK;
}

}  // namespace

// Bins every marker, sorts the columns by cell (stable) and rebuilds cell_start.
int mic_bin_and_sort(mic_ctx *ctx, int64_t *n_out) {
  const int64_t n = ctx->n;
  cudaMemsetAsync(&ctx->d_status->n_out, 0, sizeof(unsigned long long), ctx->stream);
  if (n == 0) {
    MIC_CUDA_TRY(cudaMemsetAsync(ctx->cell_start, 0, sizeof(int) * ((size_t)ctx->ncells + 2), ctx->stream));
    MIC_CUDA_TRY(cudaMemsetAsync(ctx->quad_start, 0, sizeof(int) * (4 * (size_t)ctx->ncells + 5), ctx->stream));
    ctx->sorted = 1;
    if (n_out) *n_out = 0;
    return MIC_OK;
  }
  {
    MIC_KERNEL(ctx, "k_find_cells");
    k_find_cells<<<grid_for(n, tuned_block(ctx, TU_FIND_CELLS)), tuned_block(ctx, TU_FIND_CELLS), 0, ctx->stream>>>(ctx->P, ctx->f64[C_X], ctx->f64[C_Y], ctx->i32[C_CELLX],
                                                          ctx->i32[C_CELLY], ctx->i32[C_CPU], ctx->key, n,
                                                          ctx->d_status);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  const int ntiles = (int)((n + kTile - 1) / kTile);
  int e = ensure_sort_scratch(ctx, ntiles);
  if (e) return e;
  int bits = 1;
  while ((1LL << bits) <= 4LL * ctx->ncells) ++bits;
  const int passes = (bits + kRadixBits - 1) / kRadixBits;
  int *kin = ctx->key, *kout = ctx->key_alt, *vin = ctx->perm, *vout = ctx->perm_alt;
  for (int p = 0; p < passes; ++p) {
    const int shift = p * kRadixBits;
    {
      MIC_KERNEL(ctx, "k_radix_hist");
      k_radix_hist<<<ntiles, kSortThreads, 0, ctx->stream>>>(kin, n, shift, ctx->hist, ntiles);
    }
    MIC_CUDA_TRY(cudaGetLastError());
    e = scan_exclusive(ctx, ctx->hist, (int64_t)kBuckets * ntiles, ctx->scan_aux);
    if (e) return e;
    {
      MIC_KERNEL(ctx, "k_radix_scatter");
      k_radix_scatter<<<ntiles, kSortThreads, 0, ctx->stream>>>(kin, vin, p == 0, kout, vout, n, shift, ctx->hist,
                                                                ntiles);
    }
    MIC_CUDA_TRY(cudaGetLastError());
    int *t = kin;
    kin = kout;
    kout = t;
    t = vin;
    vin = vout;
    vout = t;
  }
  // kin / vin now hold the sorted keys and the permutation
  {
    MIC_KERNEL(ctx, "k_cell_start");
    k_cell_start<<<grid_for(4LL * ctx->ncells + 5), kBlock, 0, ctx->stream>>>(kin, n, ctx->ncells,
                                                                              ctx->cell_start, ctx->quad_start);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  GatherCols g;
  g.nf = ctx->has_grain ? C_F64_COUNT : C_AOS_F64;
  for (int c = 0; c < C_F64_COUNT; ++c) {
    g.src_f[c] = ctx->f64[c];
    g.dst_f[c] = ctx->f64_alt[c];
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    g.src_i[c] = ctx->i32[c];
    g.dst_i[c] = ctx->i32_alt[c];
  }
  {
    MIC_KERNEL(ctx, "k_reorder");
    k_reorder<true><<<grid_for(n, tuned_block(ctx, TU_REORDER)), tuned_block(ctx, TU_REORDER), 0, ctx->stream>>>(
        g, vin, n, ctx->P, geo_out(ctx));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  for (int c = 0; c < g.nf; ++c) {
    double *t = ctx->f64[c];
    ctx->f64[c] = ctx->f64_alt[c];
    ctx->f64_alt[c] = t;
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    int *t = ctx->i32[c];
    ctx->i32[c] = ctx->i32_alt[c];
    ctx->i32_alt[c] = t;
  }
  ctx->sorted = 1;
  ctx->geo_valid = 1;  // computed by the gather
  if (n_out) {
    MIC_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *n_out = (int64_t)ctx->h_status->n_out;
  }
  return MIC_OK;
}

// exclusive prefix sum of data[0, len) in place; aux: mic_scan_aux_ints(len) ints of scratch
int mic_scan_exclusive(mic_ctx *ctx, int *data, int64_t len, int *aux) { return scan_exclusive(ctx, data, len, aux); }

int64_t mic_scan_aux_ints(int64_t len) {
  int64_t aux = 0, l = len;
  while (l > 1) {
    l = (l + kScanBlock - 1) / kScanBlock;
    aux += l + 1;
  }
  return aux + 16;
}

// Columns [0, n) back to the caller's marker order (slot k holds caller marker k); slots
// [n, cap) keep their contents.  The next pass bins and sorts again.
int mic_restore_caller_order(mic_ctx *ctx) {
  const int64_t cap = ctx->cap;
  if (cap == 0) return MIC_OK;
  {
    MIC_KERNEL(ctx, "k_restore_perm");
    k_restore_perm<<<grid_for(cap), kBlock, 0, ctx->stream>>>(ctx->i32[C_ID], ctx->n, cap, ctx->perm);
  }
  GatherCols g;
  g.nf = ctx->has_grain ? C_F64_COUNT : C_AOS_F64;
  for (int c = 0; c < C_F64_COUNT; ++c) {
    g.src_f[c] = ctx->f64[c];
    g.dst_f[c] = ctx->f64_alt[c];
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    g.src_i[c] = ctx->i32[c];
    g.dst_i[c] = ctx->i32_alt[c];
  }
  {
    MIC_KERNEL(ctx, "k_reorder");
    k_reorder<false><<<grid_for(cap), kBlock, 0, ctx->stream>>>(g, ctx->perm, cap, ctx->P, GeoOut{});
  }
  MIC_CUDA_TRY(cudaGetLastError());
  for (int c = 0; c < g.nf; ++c) {
    double *t = ctx->f64[c];
    ctx->f64[c] = ctx->f64_alt[c];
    ctx->f64_alt[c] = t;
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    int *t = ctx->i32[c];
    ctx->i32[c] = ctx->i32_alt[c];
    ctx->i32_alt[c] = t;
  }
  mic_invalidate_sort(ctx);
  return MIC_OK;
}

int mic_ensure_sorted(mic_ctx *ctx) {
  if (ctx->sorted) return MIC_OK;
  return mic_bin_and_sort(ctx, nullptr);
}

extern "C" int mic_find_marker_cells(mic_ctx *ctx, int64_t *n_out) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  int64_t no = 0;
  int e = mic_bin_and_sort(ctx, &no);
  if (n_out) *n_out = no;
  return e;
}

// ---- binning and stable sort for callers that cannot allocate ------------------------
//
// Some callers of this code cannot call cudaMalloc: a host that has finished its
// start-up and forbids device allocation afterwards (fixed-memory production runs),
// code that runs between the capture calls of a stream it does not own, or a plug-in
// whose host application owns the allocator.  mic_bin_sort_noalloc serves them: the
// caller passes device pointers for its inputs and outputs, and the sort's scratch (keys,
// the second value buffer, the digit histograms and the scan's block totals) lives in the
// file-scope device array below, reserved once when the library loads on a device and
// held until the process exits.  Every call shares that array, so calls whose work
// overlaps on the GPU (different streams, or different host threads on one device) race
// and must be ordered by the caller.

#include <mutex>

namespace {

constexpr int64_t kNoallocMaxMarkers = MIC_NOALLOC_MAX_MARKERS;
constexpr int64_t kNoallocMaxCells = MIC_NOALLOC_MAX_CELLS;
constexpr int64_t kNoallocTiles = (kNoallocMaxMarkers + kTile - 1) / kTile;
constexpr int64_t kNoallocHist = (int64_t)kBuckets * kNoallocTiles;
// block totals of every scan level of the histogram matrix, with one spare entry per level
constexpr int64_t kNoallocAux = (kNoallocHist + kScanBlock - 1) / kScanBlock + 64;
// layout (in 4-byte words): key | key_alt | val_alt | hist | aux, then one 8-byte counter
constexpr int64_t kOffKey = 0;
constexpr int64_t kOffKeyAlt = kOffKey + kNoallocMaxMarkers;
constexpr int64_t kOffValAlt = kOffKeyAlt + kNoallocMaxMarkers;
constexpr int64_t kOffHist = kOffValAlt + kNoallocMaxMarkers;
constexpr int64_t kOffAux = kOffHist + kNoallocHist;
constexpr int64_t kWords = (kOffAux + kNoallocAux + 63) / 64 * 64;
constexpr size_t kNoallocBytes = (size_t)kWords * 4 + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// host-side: device address of g_noalloc_scratch per CUDA context (the symbol itself is only a
// host stand-in and must never be handed to a kernel).  The cache is keyed on the context's
// process-unique id, not on the device ordinal: after cudaDeviceReset, or under another context
// of the same device, the address is looked up again instead of reusing a stale one.
std::mutex g_noalloc_mu;
constexpr int kNoallocCache = 64;
unsigned long long g_noalloc_ctx[kNoallocCache];  // context ids (0 = empty slot)
unsigned char *g_noalloc_ptr[kNoallocCache];
int g_noalloc_next;  // next slot to fill (round robin once all are used)

// the current context's id through the driver entry points (no link against libcuda); 0 when
// they are unavailable, and then the address is looked up on every call
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
    cudaGetLastError();
  });
  void *ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

__global__ void k_find_cells_grid(const double *__restrict__ X, const double *__restrict__ Y,
                                  const double *__restrict__ xg, const double *__restrict__ yg, int NX, int NY,
                                  double LX, double LY, int *__restrict__ cellX, int *__restrict__ cellY,
                                  int *__restrict__ key, int64_t n, unsigned long long *n_out) {
  __shared__ unsigned long long s_out;
  if (threadIdx.x == 0) s_out = 0;
  __syncthreads();
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < n) {
    const long long ux = nonneg_bits(X[m]), uy = nonneg_bits(Y[m]);
    const bool in = ux >= 0 && uy >= 0 && ux <= dbits(LX) && uy <= dbits(LY);
    int cx = -1, cy = -1, k = 4 * (NX - 1) * (NY - 1);
    if (in) {
      int lo = 0, hi = NX - 1;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (ux >= nonneg_bits(xg[mid])) lo = mid; else hi = mid;
      }
      cx = lo;
      lo = 0;
      hi = NY - 1;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (uy >= nonneg_bits(yg[mid])) lo = mid; else hi = mid;
      }
      cy = lo;
      // quadrant of the cell: the same test as the context binning (cell centres from x, y)
      const int qx = ux >= nonneg_bits((xg[cx] + xg[cx + 1]) / 2.0);
      const int qy = uy >= nonneg_bits((yg[cy] + yg[cy + 1]) / 2.0);
      k = 4 * (cy * (NX - 1) + cx) + 2 * qy + qx;
    } else {
      atomicAdd(&s_out, 1ULL);
    }
    cellX[m] = cx;
    cellY[m] = cy;
    key[m] = k;
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_out) atomicAdd(n_out, s_out);
}

// Device address of the scratch array in the current context.  The first call in a context
// (on each device, with that device current) looks it up with cudaGetSymbolAddress, which also
// makes the runtime set the context up; later calls in the same context reuse it.
int noalloc_scratch(unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long id = current_context_id();
  if (id)
    for (int k = 0; k < kNoallocCache; ++k)
      if (g_noalloc_ctx[k] == id) {
        *out = g_noalloc_ptr[k];
        return MIC_OK;
      }
  unsigned char *p = nullptr;
  if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess || !p) {
    cudaGetLastError();
    return MIC_ERR_CUDA;
  }
  // the lookup may have created the context: take its id now
  const unsigned long long id2 = id ? id : current_context_id();
  if (id2) {
    g_noalloc_ctx[g_noalloc_next] = id2;
    g_noalloc_ptr[g_noalloc_next] = p;
    g_noalloc_next = (g_noalloc_next + 1) % kNoallocCache;
  }
  *out = p;
  return MIC_OK;
}

}  // namespace

extern "C" int mic_bin_sort_noalloc(const double *X, const double *Y, int64_t n, const double *x, const double *y,
                                    int NX, int NY, double LX, double LY, int32_t *cellX, int32_t *cellY,
                                    int32_t *perm, int32_t *cell_start, void *stream, int64_t *n_out) {
  if (n < 0 || NX < 3 || NY < 3 || !x || !y || !cell_start) return MIC_ERR_ARG;
  if (n > 0 && (!X || !Y || !cellX || !cellY || !perm)) return MIC_ERR_ARG;
  if (n > kNoallocMaxMarkers) return MIC_ERR_CAPACITY;
  const int64_t ncells = (int64_t)(NX - 1) * (NY - 1);
  if (ncells > kNoallocMaxCells) return MIC_ERR_CAPACITY;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return MIC_ERR_NO_DEVICE;
  unsigned char *base = nullptr;
  int e = noalloc_scratch(&base);
  if (e) return e;
  cudaStream_t s = (cudaStream_t)stream;
  int *words = reinterpret_cast<int *>(base);
  int *key = words + kOffKey, *key_alt = words + kOffKeyAlt, *val_alt = words + kOffValAlt;
  int *hist = words + kOffHist, *aux = words + kOffAux;
  unsigned long long *d_out = reinterpret_cast<unsigned long long *>(base + (size_t)kWords * 4);
  // the counter keeps the previous call's value: clear it
  if (cudaMemsetAsync(d_out, 0, sizeof(unsigned long long), s) != cudaSuccess) return MIC_ERR_CUDA;
  if (n > 0) {
    k_find_cells_grid<<<grid_for(n), kBlock, 0, s>>>(X, Y, x, y, NX, NY, LX, LY, cellX, cellY, key, n, d_out);
    if (cudaGetLastError() != cudaSuccess) return MIC_ERR_CUDA;
    const int ntiles = (int)((n + kTile - 1) / kTile);
    int bits = 1;
    while ((1LL << bits) <= 4 * ncells) ++bits;
    const int passes = (bits + kRadixBits - 1) / kRadixBits;
    // the last pass must write the caller's perm[]: pick the ping-pong order accordingly
    int *vbuf[2] = {(passes & 1) ? perm : val_alt, (passes & 1) ? val_alt : perm};
    int *kbuf[2] = {key_alt, key};
    int *kin = key, *vin = nullptr;
    for (int p = 0; p < passes; ++p) {
      int *kout = kbuf[p & 1], *vout = vbuf[p & 1];
      k_radix_hist<<<ntiles, kSortThreads, 0, s>>>(kin, n, p * kRadixBits, hist, ntiles);
      if (cudaGetLastError() != cudaSuccess) return MIC_ERR_CUDA;
      // every bucket of every tile is written by k_radix_hist, so nothing stale survives
      const int64_t len = (int64_t)kBuckets * ntiles;
      const int64_t nb = (len + kScanBlock - 1) / kScanBlock;
      if (nb <= 1) {
        k_scan_block<<<1, kScanThreads, 0, s>>>(hist, len, nullptr);
      } else {
        // two levels suffice: nb <= kScanBlock for the largest histogram matrix
        k_scan_block<<<(unsigned)nb, kScanThreads, 0, s>>>(hist, len, aux);
        k_scan_block<<<1, kScanThreads, 0, s>>>(aux, nb, nullptr);
        k_scan_add<<<(unsigned)nb, kScanThreads, 0, s>>>(hist, len, aux);
      }
      k_radix_scatter<<<ntiles, kSortThreads, 0, s>>>(kin, vin, p == 0, kout, vout, n, p * kRadixBits, hist,
                                                       ntiles);
      if (cudaGetLastError() != cudaSuccess) return MIC_ERR_CUDA;
      kin = kout;
      vin = vout;
    }
    k_cell_start<<<grid_for(4LL * ncells + 5), kBlock, 0, s>>>(kin, n, (int)ncells, cell_start, nullptr);
  } else {
    if (cudaMemsetAsync(cell_start, 0, sizeof(int32_t) * (size_t)(ncells + 2), s) != cudaSuccess)
      return MIC_ERR_CUDA;
  }
  if (cudaGetLastError() != cudaSuccess) return MIC_ERR_CUDA;
  if (n_out) {
    unsigned long long h = 0;
    if (cudaMemcpyAsync(&h, d_out, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MIC_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return MIC_ERR_CUDA;
    *n_out = (int64_t)h;
  }
  return MIC_OK;
}
