// mic_density.cu -- marker density control: checkMarkerDensity (markers.c:455-781) on the device.
//
// The reference counts markers per basic quarter cell, draws drand48 numbers to pick markers
// to remove from overfull quarter cells, draws positions for markers to add to sparse ones,
// recycles out-of-domain slots last-in first-out, and gives each new marker the properties of
// its nearest neighbour (or, in the first and last cell columns, those of a subduction inflow
// marker).  Everything that decides results is reproduced; the work is split by what depends
// on what:
//   plan      one thread per quarter cell: counts are the runs of the binning's (cell,
//             quadrant) sort key, no extra pass over the markers;
//   scans     block scans give each quarter cell its slice of the additions, the removals and
//             the random stream;
//   out list  out-of-domain markers in caller order (flag per caller index + scan);
//   removal   one block per overfull quarter cell: candidates sorted by caller index, their
//             drand48 values by closed-form skip-ahead, the smallest ones removed;
//   positions one thread per quarter cell, values by skip-ahead, recycled or appended slot;
//   neighbours one warp per new marker over the static candidate set (markers that were in the
//             domain before the call and not removed);
//   fill      the only order-dependent part -- a recycled slot filled by an earlier new marker
//             becomes a candidate for later ones.  Decisions for all new markers at once from
//             estimated facts about the earlier ones, roots of the chains of copies by pointer
//             jumping, repeated until the estimates reproduce themselves; then one copy per slot.
//             A slot recycled twice (the reference's over-removal case), or no fixed point within
//             64 rounds, falls back to one warp walking the new markers in order.
// The drand48 stream (the reference's drand48() calls and its PETSCRAND48 object share it) is a
// 48-bit state kept in the context.
#include <cmath>
#include <climits>
#include <vector>

#include "mic_internal.cuh"
#include "mic_rheology.cuh"

using namespace mic;

namespace {

constexpr int kMaxCand = 2048;  // markers of one overfull quarter cell handled in shared memory

struct DCols {
  double *f[C_F64_COUNT];
  int *i[C_I32_COUNT];
};

__host__ __device__ inline unsigned long long lcg48_skip(unsigned long long x0, unsigned long long k) {
  unsigned long long A = 0x5DEECE66DULL, C = 0xBULL, m = 1ULL, a = 0ULL;
  while (k) {
    if (k & 1ULL) {
      m = A * m;
      a = A * a + C;
    }
    C = A * C + C;
    A = A * A;
    k >>= 1;
  }
  return (m * x0 + a) & 0xFFFFFFFFFFFFULL;
}

// quarter cell r in the reference's order (i fastest over 2 (NX-1), then j) -> binning key
__device__ inline void qc_ij(int r, int NX, int &i, int &j) {
  const int w = 2 * (NX - 1);
  i = r % w;
  j = r / w;
}
__device__ inline int qc_key(int i, int j, int NX) { return 4 * ((j >> 1) * (NX - 1) + (i >> 1)) + 2 * (j & 1) + (i & 1); }

// bounds of quarter cell (i, j) (markers.c:628-632, 700-710)
__device__ inline void qc_box(const Params &P, int i, int j, double &x0, double &x1, double &y0, double &y1) {
  x0 = !(i & 1) ? P.x[i / 2] : P.xc[(i + 1) / 2];
  x1 = !(i & 1) ? P.xc[i / 2 + 1] : P.x[(i + 1) / 2];
  y0 = !(j & 1) ? P.y[j / 2] : P.yc[(j + 1) / 2];
  y1 = !(j & 1) ? P.yc[j / 2 + 1] : P.y[(j + 1) / 2];
}

// findMarkerCell's bisection (markers.c:47-69) on one axis, in-domain values
__device__ inline int bisect(const double *g, int n, double v) {
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (v >= g[mid])
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// cell range that holds every point of [v - w, v + w]
__device__ inline void window(const double *g, int n, double v, double w, int &lo, int &hi) {
  lo = bisect(g, n, fmax(v - w, g[0]));
  hi = bisect(g, n, fmin(v + w, g[n - 1]));
  lo = max(lo - 1, 0);
  hi = min(hi + 1, n - 2);
}

__device__ inline double stream_u(unsigned long long s0, unsigned long long k) {
  return (double)lcg48_skip(s0, k) * (1.0 / 281474976710656.0);
}

__device__ inline bool better(double r, int id, double br, int bid) { return r < br || (r == br && id < bid); }

// ---- plan -----------------------------------------------------------------------------------

__global__ void k_density_plan(Params P, const int *__restrict__ qs, const double *__restrict__ X,
                               const double *__restrict__ Y, int nq, mic_density_options d, int *qadd, int *qrem,
                               int *qdraw, int *qflag, int *err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nq) return;
  if (r == nq) {  // totals land here after the scans
    qadd[nq] = qrem[nq] = qdraw[nq] = qflag[nq] = 0;
    return;
  }
  int i, j;
  qc_ij(r, P.NX, i, j);
  const int key = qc_key(i, j, P.NX);
  const int cnt = qs[key + 1] - qs[key];
  int add = 0, rem = 0, draws = 0;
  if (cnt < d.minMarkers) {  // markers.c:574-599
    double dy = P.y[j / 2 + 1] - P.y[j / 2];
    double dx = P.x[i / 2 + 1] - P.x[i / 2];
    dx /= 2.0;
    dy /= 2.0;
    const long long mx = (long long)ceil((double)(d.NMX * (P.NX - 1)) / 2.0 * dx / P.LX);
    const long long my = (long long)ceil((double)(d.NMY * (P.NY - 1)) / 2.0 * dy / P.LY);
    const long long mynadd = mx * my - cnt;
    if (mynadd <= 0 || mynadd > INT_MAX / 4)
      atomicOr(err, 1);
    else
      add = (int)mynadd;
  } else if (cnt > d.maxMarkers) {
    rem = cnt - d.maxMarkers;
    double x0, x1, y0, y1;
    qc_box(P, i, j, x0, x1, y0, y1);
    for (int s = qs[key]; s < qs[key + 1]; ++s)
      if (X[s] >= x0 && X[s] < x1 && Y[s] >= y0 && Y[s] < y1) ++draws;
    if (draws == 0) atomicOr(err, 2);
  }
  qadd[r] = add;
  qrem[r] = rem;
  qdraw[r] = draws;
  qflag[r] = rem > 0;
}

__global__ void k_density_ids(const int *__restrict__ cellX, const int *__restrict__ ID, int64_t n, int *slot_of_id,
                              int *outflag) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s > n) return;
  if (s == n) {
    outflag[n] = 0;
    return;
  }
  const int id = ID[s];
  slot_of_id[id] = (int)s;
  outflag[id] = cellX[s] == -1;
}

__global__ void k_density_outlist(const int *__restrict__ cellX, const int *__restrict__ slot_of_id,
                                  const int *__restrict__ outpos, int64_t n, int *isout) {
  const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (id >= n) return;
  if (cellX[slot_of_id[id]] == -1) isout[outpos[id]] = (int)id;
}

__global__ void k_density_remcells(const int *__restrict__ qflag, int nq, int *remcells) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nq && qflag[r + 1] > qflag[r]) remcells[qflag[r]] = r;
}

// ---- removal ----------------------------------------------------------------------------------

__device__ void bitonic_u64(unsigned long long *a, int n) {  // ascending, n a power of two
  for (int k = 2; k <= n; k <<= 1) {
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int p = t ^ jj;
        if (p > t) {
          const bool up = (t & k) == 0;
          const unsigned long long u = a[t], v = a[p];
          if ((u > v) == up) {
            a[t] = v;
            a[p] = u;
          }
        }
      }
      __syncthreads();
    }
  }
}

// markers.c:626-676: the run's markers inside the quarter cell's bounds, in caller order, each
// with the next drand48 value; the ones with the smallest values leave the domain
__global__ void __launch_bounds__(256) k_density_remove(Params P, const int *__restrict__ qs,
                                                        const int *__restrict__ remcells, const int *__restrict__ qrem,
                                                        const int *__restrict__ qdraw, DCols c, unsigned long long s0,
                                                        int out0, int *isout, int *err) {
  __shared__ unsigned long long cand[kMaxCand];  // (caller id << 32) | slot
  __shared__ unsigned long long pick[kMaxCand];  // (stream state << 16) | rank
  __shared__ int nc;
  const int r = remcells[blockIdx.x];
  int i, j;
  qc_ij(r, P.NX, i, j);
  const int key = qc_key(i, j, P.NX);
  double x0, x1, y0, y1;
  qc_box(P, i, j, x0, x1, y0, y1);
  if (threadIdx.x == 0) nc = 0;
  __syncthreads();
  const double *X = c.f[C_X], *Y = c.f[C_Y];
  for (int s = qs[key] + threadIdx.x; s < qs[key + 1]; s += blockDim.x) {
    if (X[s] >= x0 && X[s] < x1 && Y[s] >= y0 && Y[s] < y1) {
      const int p = atomicAdd(&nc, 1);
      if (p < kMaxCand) cand[p] = ((unsigned long long)(unsigned)c.i[C_ID][s] << 32) | (unsigned)s;
    }
  }
  __syncthreads();
  const int N = nc;
  if (N > kMaxCand || N == 0) {
    if (threadIdx.x == 0) atomicOr(err, N == 0 ? 2 : 4);
    return;
  }
  int P2 = 1;
  while (P2 < N) P2 <<= 1;
  for (int t = N + threadIdx.x; t < P2; t += blockDim.x) cand[t] = ~0ULL;
  __syncthreads();
  bitonic_u64(cand, P2);
  const unsigned long long base = (unsigned long long)qdraw[r];
  for (int t = threadIdx.x; t < P2; t += blockDim.x)
    pick[t] = t < N ? (lcg48_skip(s0, base + t + 1) << 16) | (unsigned long long)t : ~0ULL;
  __syncthreads();
  bitonic_u64(pick, P2);
  const int toRemove = qrem[r + 1] - qrem[r];
  for (int e = threadIdx.x; e < toRemove; e += blockDim.x) {
    // all candidates gone: the reference's search falls back to the first one
    const int k = e < N ? (int)(pick[e] & 0xFFFF) : 0;
    if (e >= N) err[1] = 1;  // a slot listed twice: only the in-order fill gives the reference's result
    const int slot = (int)(cand[k] & 0xFFFFFFFFULL);
    isout[out0 + qrem[r] + e] = (int)(cand[k] >> 32);
    c.f[C_X][slot] = -1.0;
    c.f[C_Y][slot] = -1.0;
    c.i[C_CELLX][slot] = -1;
    c.i[C_CELLY][slot] = -1;
  }
}

// ---- additions -----------------------------------------------------------------------------

// markers.c:689-716 (positions) and 722-731 (slot: last out-of-domain marker first, then append)
__global__ void k_density_positions(Params P, const int *__restrict__ qadd, int nq, unsigned long long s1, double plate,
                                    int nout, int64_t nmark, int64_t n, const int *__restrict__ isout,
                                    const int *__restrict__ slot_of_id, double *nx, double *ny, int *tid, int *tslot,
                                    int *kind) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nq) return;
  const int cnt = qadd[r + 1] - qadd[r];
  if (cnt == 0) return;
  int i, j;
  qc_ij(r, P.NX, i, j);
  double x0, x1, y0, y1;
  qc_box(P, i, j, x0, x1, y0, y1);
  for (int k = 0; k < cnt; ++k) {
    const long long t = qadd[r] + k;
    const double ux = stream_u(s1, 2ULL * t + 1ULL), uy = stream_u(s1, 2ULL * t + 2ULL);
    const double xv = __dadd_rn(x0, __dmul_rn(__dsub_rn(x1, x0), ux));
    const double yv = __dadd_rn(y0, __dmul_rn(__dsub_rn(y1, y0), uy));
    nx[t] = xv;
    ny[t] = yv;
    kind[t] = (xv < P.x[1]) ? 1 : ((xv >= P.x[P.NX - 2] && yv >= plate) ? 2 : 0);
    if (t < nout) {
      const int id = isout[nout - 1 - t];
      tid[t] = id;
      tslot[t] = slot_of_id[id];
    } else {
      tid[t] = (int)(nmark + (t - nout));
      tslot[t] = (int)(n + (t - nout));
    }
  }
}

// markers.c:740-760 over the markers that were in the domain before the call and were not
// removed: one warp per new marker, nearest by (distance, caller index)
__global__ void k_density_nn(Params P, const int *__restrict__ cell_start, DCols c, const double *__restrict__ nx,
                             const double *__restrict__ ny, const int *__restrict__ kind, int nadd, double wmax,
                             double hmax, double mind0, double *best_r, int *best_id, int *best_slot) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= nadd) return;
  double br = mind0;
  int bid = INT_MAX, bs = -1;
  if (kind[t] == 0) {
    const double xv = nx[t], yv = ny[t];
    int cx0, cx1, cy0, cy1;
    window(P.x, P.NX, xv, wmax, cx0, cx1);
    window(P.y, P.NY, yv, hmax, cy0, cy1);
    for (int cy = cy0; cy <= cy1; ++cy) {
      for (int cx = cx0; cx <= cx1; ++cx) {
        const int cell = cy * (P.NX - 1) + cx;
        for (int s = cell_start[cell] + lane; s < cell_start[cell + 1]; s += 32) {
          const int mx = c.i[C_CELLX][s];
          if (mx == -1) continue;
          const int my = c.i[C_CELLY][s];
          const double xm = c.f[C_X][s], ym = c.f[C_Y][s];
          if (fabs(xm - xv) <= (P.x[mx + 1] - P.x[mx]) && fabs(ym - yv) <= (P.y[my + 1] - P.y[my])) {
            const double x1 = xm - xv, y1 = ym - yv;
            const double r1 = sqrt(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)));
            const int id = c.i[C_ID][s];
            if (r1 < mind0 && better(r1, id, br, bid)) {
              br = r1;
              bid = id;
              bs = s;
            }
          }
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double r2 = __shfl_down_sync(0xffffffffu, br, o);
      const int i2 = __shfl_down_sync(0xffffffffu, bid, o), s2 = __shfl_down_sync(0xffffffffu, bs, o);
      if (better(r2, i2, br, bid)) {
        br = r2;
        bid = i2;
        bs = s2;
      }
    }
  }
  if (lane == 0) {
    best_r[t] = br;
    best_id[t] = bid;
    best_slot[t] = bs;
  }
}

// new_slab_marker / new_inflow_marker (benchmarkInitialConditions.c:44-66) + findMarkerCell into
// slot; cpu and the strain-rate residual, which the reference leaves uninitialised, are 0
__device__ void build_inflow_marker(const Params &P, const mic_materials &M, const mic_options &O,
                                    const CreepConfig &cfg, const DCols &c, int nf, const mic_density_options &d,
                                    int kind, double xv, double yv, int slot) {
  for (int f = 0; f < nf; ++f) c.f[f][slot] = 0.0;
  if (nf > C_GRAIN) c.f[C_GRAIN][slot] = kGrainArgDefault;
  for (int f = 0; f < C_I32_COUNT; ++f)
    if (f != C_ID) c.i[f][slot] = 0;
  double T;
  if (kind == 1) {  // slab_inflow_temperature (benchmarkInitialConditions.c:124-134)
    const double slab_age_s = d.slabAge * 1.0e6 * 3.15576e7;
    T = 273.0 + (1623.0 - 273.0) * erf((yv - xv * tan(d.slabAngle)) / (2.0 * sqrt(0.7272e-6 * slab_age_s)));
  } else {
    T = 1573.0;  // mantle_temperature
  }
  c.f[C_X][slot] = xv;
  c.f[C_Y][slot] = yv;
  c.f[C_T][slot] = T;
  c.i[C_MAT][slot] = 0;
  double eta, mu;
  CreepIn ci = {0.0, 0.0, 0.0, kGrainArgDefault, 0.0, 0.0f, 0, 0, 0.0, 0, {}, 0.0};
  CreepConfig exact = cfg;
  exact.mode = 0;
  if (rheology(M, O, 0, T, xv, yv, eta, mu, &exact, &ci)) {
    c.f[C_ETA][slot] = eta;
    c.f[C_MU][slot] = mu;
  }
  const bool in = xv >= 0.0 && yv >= 0.0 && xv <= P.LX && yv <= P.LY;
  c.i[C_CELLX][slot] = in ? bisect(P.x, P.NX, xv) : -1;
  c.i[C_CELLY][slot] = in ? bisect(P.y, P.NY, yv) : -1;
}

// cell holding a (clamped) position
__device__ __forceinline__ int pos_cell(const Params &P, double xv, double yv) {
  return bisect(P.y, P.NY, fmin(fmax(yv, P.y[0]), P.y[P.NY - 1])) * (P.NX - 1) +
         bisect(P.x, P.NX, fmin(fmax(xv, P.x[0]), P.x[P.NX - 1]));
}

// ---- parallel fill ------------------------------------------------------------------------
// Taken in order, new marker t copies the nearest of the static candidates and of the recycled
// slots that earlier new markers t' < t filled inside its window.  A copy keeps its source's cell
// until the next binning, so the window test of a later marker against t' uses the cell of t''s
// root: the static or inflow marker at the start of its chain of copies.  Three facts about t'
// enter later decisions: whether it was filled, its root's cell and its position (known).  The
// facts are estimated for every t' at once, every decision is taken from the estimates, roots are
// found by pointer jumping and the facts recomputed.  Decisions look only backwards, so estimates
// that reproduce themselves give the in-order result (by induction over t); each slot then takes
// its root's columns and its own position.

__global__ void k_density_bucket(Params P, const double *__restrict__ nx, const double *__restrict__ ny, int nrec,
                                 int *tcell, int *ccount) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrec) return;
  const int cell = pos_cell(P, nx[t], ny[t]);
  tcell[t] = cell;
  atomicAdd(&ccount[cell], 1);
}

__global__ void k_density_scatter(const int *__restrict__ tcell, const int *__restrict__ cstart, int nrec, int *cfill,
                                  int *clist) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrec) return;
  const int cell = tcell[t];
  clist[cstart[cell] + atomicAdd(&cfill[cell], 1)] = t;
}

// first estimates: every new marker filled, its root in its own cell
__global__ void k_density_guess(Params P, const double *__restrict__ nx, const double *__restrict__ ny, int nadd,
                                int *ewrote, int *ecx, int *ecy) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nadd) return;
  ewrote[t] = 1;
  ecx[t] = bisect(P.x, P.NX, fmin(fmax(nx[t], P.x[0]), P.x[P.NX - 1]));
  ecy[t] = bisect(P.y, P.NY, fmin(fmax(ny[t], P.y[0]), P.y[P.NY - 1]));
}

// markers.c:740-760 for new marker t against the recycled slots of earlier new markers, with the
// estimated facts; the static candidates' best is already known
__global__ void k_density_decide(Params P, const double *__restrict__ nx, const double *__restrict__ ny,
                                 const int *__restrict__ kind, const int *__restrict__ tid,
                                 const double *__restrict__ best_r, const int *__restrict__ best_id,
                                 const int *__restrict__ cstart, const int *__restrict__ clist, int nadd, double wmax,
                                 double hmax, const int *__restrict__ ewrote, const int *__restrict__ ecx,
                                 const int *__restrict__ ecy, int *src, int *ptr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nadd) return;
  int bt = -1;
  if (kind[t] == 0) {
    const int id = tid[t];
    const double xv = nx[t], yv = ny[t];
    double br = best_r[t];
    int bid = best_id[t];
    int cx0, cx1, cy0, cy1;
    window(P.x, P.NX, xv, wmax, cx0, cx1);
    window(P.y, P.NY, yv, hmax, cy0, cy1);
    for (int cy = cy0; cy <= cy1; ++cy)
      for (int cx = cx0; cx <= cx1; ++cx) {
        const int cell = cy * (P.NX - 1) + cx;
        for (int e = cstart[cell]; e < cstart[cell + 1]; ++e) {
          const int t2 = clist[e];
          if (t2 >= t || !ewrote[t2]) continue;
          const int id2 = tid[t2];
          const int mx = ecx[t2], my = ecy[t2];
          if (id2 == id || mx == -1) continue;
          const double xm = nx[t2], ym = ny[t2];
          if (fabs(xm - xv) <= (P.x[mx + 1] - P.x[mx]) && fabs(ym - yv) <= (P.y[my + 1] - P.y[my])) {
            const double x1 = xm - xv, y1 = ym - yv;
            const double r1 = sqrt(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)));
            if (better(r1, id2, br, bid)) {
              br = r1;
              bid = id2;
              bt = t2;
            }
          }
        }
      }
  }
  src[t] = bt;
  ptr[t] = bt >= 0 ? bt : t;
}

__global__ void k_density_jump(const int *__restrict__ in, int *out, int nadd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nadd) out[t] = in[in[t]];
}

// the facts the decisions imply: filled, root cell, root slot; any change from the estimates
// means another round
__global__ void k_density_facts(Params P, DCols c, const double *__restrict__ nx, const double *__restrict__ ny,
                                const int *__restrict__ kind, const int *__restrict__ tslot,
                                const int *__restrict__ best_slot, const int *__restrict__ src,
                                const int *__restrict__ root, int nadd, int *ewrote, int *ecx, int *ecy, int *rslot,
                                int *changed) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nadd) return;
  const int r = root[t];
  int w = 0, cx = -1, cy = -1, rs = -1;
  if (kind[r] != 0) {  // inflow marker: findMarkerCell of its own position
    const double xv = nx[r], yv = ny[r];
    const bool in = xv >= 0.0 && yv >= 0.0 && xv <= P.LX && yv <= P.LY;
    w = 1;
    cx = in ? bisect(P.x, P.NX, xv) : -1;
    cy = in ? bisect(P.y, P.NY, yv) : -1;
    rs = tslot[r];
  } else if (best_slot[r] >= 0) {
    rs = best_slot[r];
    w = 1;
    cx = c.i[C_CELLX][rs];
    cy = c.i[C_CELLY][rs];
  }
  if (src[t] >= 0) w = 1;
  rslot[t] = rs;
  if (w != ewrote[t] || cx != ecx[t] || cy != ecy[t]) {
    ewrote[t] = w;
    ecx[t] = cx;
    ecy[t] = cy;
    *changed = 1;
  }
}

__global__ void k_density_build(Params P, mic_materials M, mic_options O, CreepConfig cfg, DCols c, int nf,
                                mic_density_options d, const double *__restrict__ nx, const double *__restrict__ ny,
                                const int *__restrict__ kind, const int *__restrict__ tid,
                                const int *__restrict__ tslot, int nadd, int64_t nmark) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nadd || kind[t] == 0) return;
  build_inflow_marker(P, M, O, cfg, c, nf, d, kind[t], nx[t], ny[t], tslot[t]);
  if (tid[t] >= nmark) c.i[C_ID][tslot[t]] = tid[t];
}

// markers[idx] = markers[minidx] with the new position (markers.c:761-764); the source's columns
// are its root's
__global__ void k_density_copy(DCols c, int nf, const double *__restrict__ nx, const double *__restrict__ ny,
                               const int *__restrict__ kind, const int *__restrict__ tid,
                               const int *__restrict__ tslot, const int *__restrict__ ewrote,
                               const int *__restrict__ rslot, int nadd, int64_t nmark) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nadd || kind[t] != 0) return;
  const int slot = tslot[t], rs = rslot[t];
  if (ewrote[t] && rs >= 0) {
    for (int f = 0; f < nf; ++f) c.f[f][slot] = c.f[f][rs];
    for (int f = 0; f < C_I32_COUNT; ++f)
      if (f != C_ID) c.i[f][slot] = c.i[f][rs];
    c.f[C_X][slot] = nx[t];
    c.f[C_Y][slot] = ny[t];
  }
  if (tid[t] >= nmark) c.i[C_ID][slot] = tid[t];
}

// one warp, new markers in order (markers.c:720-765)
__global__ void k_density_fill(Params P, mic_materials M, mic_options O, CreepConfig cfg, DCols c, int nf,
                               mic_density_options d, const double *__restrict__ nx, const double *__restrict__ ny,
                               const int *__restrict__ kind, const int *__restrict__ tid, const int *__restrict__ tslot,
                               const double *__restrict__ best_r, const int *__restrict__ best_id,
                               const int *__restrict__ best_slot, int nadd, int64_t nmark, double wmax, double hmax,
                               int *heads, int *next) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x >= 32) return;
  for (int t = 0; t < nadd; ++t) {
    const int id = tid[t], slot = tslot[t];
    const double xv = nx[t], yv = ny[t];
    bool wrote = false;
    if (kind[t] != 0) {
      if (lane == 0) build_inflow_marker(P, M, O, cfg, c, nf, d, kind[t], xv, yv, slot);
      wrote = true;
    } else {
      double br = best_r[t];
      int bid = best_id[t], bs = best_slot[t];
      int cx0, cx1, cy0, cy1;
      window(P.x, P.NX, xv, wmax, cx0, cx1);
      window(P.y, P.NY, yv, hmax, cy0, cy1);
      const int wx = cx1 - cx0 + 1, ncell = wx * (cy1 - cy0 + 1);
      for (int q = lane; q < ncell; q += 32) {  // recycled slots filled earlier in this call
        const int cell = (cy0 + q / wx) * (P.NX - 1) + cx0 + q % wx;
        for (int e = heads[cell]; e != -1; e = next[e]) {
          const int s2 = tslot[e], id2 = tid[e];
          if (id2 == id) continue;
          const int mx = c.i[C_CELLX][s2], my = c.i[C_CELLY][s2];
          if (mx == -1) continue;
          const double xm = c.f[C_X][s2], ym = c.f[C_Y][s2];
          if (fabs(xm - xv) <= (P.x[mx + 1] - P.x[mx]) && fabs(ym - yv) <= (P.y[my + 1] - P.y[my])) {
            const double x1 = xm - xv, y1 = ym - yv;
            const double r1 = sqrt(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)));
            if (better(r1, id2, br, bid)) {
              br = r1;
              bid = id2;
              bs = s2;
            }
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffffu, br, o);
        const int i2 = __shfl_down_sync(0xffffffffu, bid, o), s2 = __shfl_down_sync(0xffffffffu, bs, o);
        if (better(r2, i2, br, bid)) {
          br = r2;
          bid = i2;
          bs = s2;
        }
      }
      bs = __shfl_sync(0xffffffffu, bs, 0);
      if (bs >= 0) {  // markers[idx] = markers[minidx], then the new position
        for (int f = lane; f < nf; f += 32) c.f[f][slot] = c.f[f][bs];
        if (lane < C_I32_COUNT && lane != C_ID) c.i[lane][slot] = c.i[lane][bs];
        __syncwarp();
        if (lane == 0) {
          c.f[C_X][slot] = xv;
          c.f[C_Y][slot] = yv;
        }
        wrote = true;
      }
    }
    if (lane == 0) {
      if (id >= nmark) c.i[C_ID][slot] = id;  // appended slot
      if (wrote && id < nmark) {  // a recycled slot joins the candidates of later new markers
        const int cell = pos_cell(P, xv, yv);
        next[t] = heads[cell];
        heads[cell] = t;
      }
    }
    __syncwarp();
  }
}

struct Totals {
  int nadd, nrem, ndraw, nremcells, nout;
};

__global__ void k_density_totals(const int *qadd, const int *qrem, const int *qdraw, const int *qflag, int nq,
                                 const int *outflag, int64_t n, Totals *t) {
  t->nadd = qadd[nq];
  t->nrem = qrem[nq];
  t->ndraw = qdraw[nq];
  t->nremcells = qflag[nq];
  t->nout = outflag[n];
}

template <typename T>
T *carve(unsigned char *&p, int64_t count) {
  T *r = reinterpret_cast<T *>(p);
  p += ((count * (int64_t)sizeof(T) + 255) / 256) * 256;
  return r;
}

int ensure_buf(void **buf, size_t *have, size_t need) {
  if (*have >= need) return MIC_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  if (cudaMalloc(buf, need) != cudaSuccess) return MIC_ERR_NOMEM;
  *have = need;
  return MIC_OK;
}

}  // namespace

extern "C" int mic_density_seed(mic_ctx *ctx, long seed) {
  if (!ctx) return MIC_ERR_ARG;
  ctx->rng48 = ((unsigned long long)(seed & 0xFFFFFFFFL) << 16) | 0x330EULL;
  return MIC_OK;
}

extern "C" int mic_density_rng_state(mic_ctx *ctx, uint64_t *get, const uint64_t *set) {
  if (!ctx) return MIC_ERR_ARG;
  if (get) *get = ctx->rng48;
  if (set) ctx->rng48 = *set & 0xFFFFFFFFFFFFULL;
  return MIC_OK;
}

extern "C" int mic_density_fill_rounds(mic_ctx *ctx, int *rounds) {
  if (!ctx || !rounds) return MIC_ERR_ARG;
  *rounds = ctx->density_rounds;
  return MIC_OK;
}

extern "C" int mic_check_marker_density(mic_ctx *ctx, const mic_density_options *d, int64_t *n_added,
                                        int64_t *n_removed) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !d || d->NMX < 1 || d->NMY < 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n_added) *n_added = 0;
  if (n_removed) *n_removed = 0;
  ctx->density_rounds = 0;
  int e = mic_ensure_sorted(ctx);  // cells of the current positions (findMarkerCells, main:247)
  if (e) return e;
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const int nq = 4 * ctx->ncells;
  const int64_t n = ctx->n, cap = ctx->cap;
  // ---- plan, out-of-domain list, scans ----
  const int64_t aux_q = mic_scan_aux_ints(nq + 1), aux_n = mic_scan_aux_ints(n + 1);
  size_t need = 0;
  need += 4 * (((nq + 1) * sizeof(int) + 255) / 256) * 256;                              // qadd qrem qdraw qflag
  need += ((nq * sizeof(int) + 255) / 256) * 256;                                       // remcells
  need += ((((n + 1) > 0 ? n + 1 : 1) * sizeof(int) + 255) / 256) * 256 * 2;             // outflag, slot_of_id
  need += (((2 * n + 2 * (int64_t)nq + 1) * sizeof(int) + 255) / 256) * 256;            // isout
  need += (((aux_q > aux_n ? aux_q : aux_n) * sizeof(int) + 255) / 256) * 256;          // scan scratch
  need += 256 + ((ctx->ncells * sizeof(int) + 255) / 256) * 256 + 256;                    // totals, heads
  if ((e = ensure_buf(&ctx->dens_buf, &ctx->dens_bytes, need))) return e;
  unsigned char *p = (unsigned char *)ctx->dens_buf;
  int *qadd = carve<int>(p, nq + 1), *qrem = carve<int>(p, nq + 1), *qdraw = carve<int>(p, nq + 1);
  int *qflag = carve<int>(p, nq + 1), *remcells = carve<int>(p, nq);
  int *outflag = carve<int>(p, n + 1), *slot_of_id = carve<int>(p, n + 1);
  int *isout = carve<int>(p, 2 * n + 2 * (int64_t)nq + 1);
  int *aux = carve<int>(p, aux_q > aux_n ? aux_q : aux_n);
  Totals *tot = carve<Totals>(p, 1);
  int *err = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(tot) + 128);
  int *heads = carve<int>(p, ctx->ncells);
  MIC_CUDA_TRY(cudaMemsetAsync(err, 0, 2 * sizeof(int), ctx->stream));
  DCols c;
  for (int k = 0; k < C_F64_COUNT; ++k) c.f[k] = ctx->f64[k];
  for (int k = 0; k < C_I32_COUNT; ++k) c.i[k] = ctx->i32[k];
  {
    MIC_KERNEL(ctx, "k_density_plan");
    k_density_plan<<<grid_for(nq + 1), kBlock, 0, ctx->stream>>>(ctx->P, ctx->quad_start, ctx->f64[C_X],
                                                                  ctx->f64[C_Y], nq, *d, qadd, qrem, qdraw, qflag, err);
  }
  {
    MIC_KERNEL(ctx, "k_density_ids");
    k_density_ids<<<grid_for(n + 1), kBlock, 0, ctx->stream>>>(ctx->i32[C_CELLX], ctx->i32[C_ID], n, slot_of_id,
                                                                outflag);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  int *scans[4] = {qadd, qrem, qdraw, qflag};
  for (int k = 0; k < 4; ++k)
    if ((e = mic_scan_exclusive(ctx, scans[k], nq + 1, aux))) return e;
  if ((e = mic_scan_exclusive(ctx, outflag, n + 1, aux))) return e;
  if (n > 0) {
    MIC_KERNEL(ctx, "k_density_outlist");
    k_density_outlist<<<grid_for(n), kBlock, 0, ctx->stream>>>(ctx->i32[C_CELLX], slot_of_id, outflag, n, isout);
  }
  {
    MIC_KERNEL(ctx, "k_density_remcells");
    k_density_remcells<<<grid_for(nq), kBlock, 0, ctx->stream>>>(qflag, nq, remcells);
  }
  {
    MIC_KERNEL(ctx, "k_density_totals");
    k_density_totals<<<1, 1, 0, ctx->stream>>>(qadd, qrem, qdraw, qflag, nq, outflag, n, tot);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  Totals h;
  int herr[2] = {0, 0};
  MIC_CUDA_TRY(cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaMemcpyAsync(herr, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (herr[0]) return MIC_ERR_DENSITY;
  // ---- removal ----
  const unsigned long long s0 = ctx->rng48;
  if (h.nrem > 0) {
    {
      MIC_KERNEL(ctx, "k_density_remove");
      k_density_remove<<<h.nremcells, 256, 0, ctx->stream>>>(ctx->P, ctx->quad_start, remcells, qrem, qdraw, c, s0,
                                                             h.nout, isout, err);
    }
    MIC_CUDA_TRY(cudaGetLastError());
    MIC_CUDA_TRY(cudaMemcpyAsync(herr, err, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (herr[0]) return MIC_ERR_DENSITY;
    if (n_removed) *n_removed = h.nrem;
  }
  const unsigned long long s1 = lcg48_skip(s0, (unsigned long long)h.ndraw);
  ctx->rng48 = s1;
  mic_invalidate_sort(ctx);
  const int64_t nout = (int64_t)h.nout + h.nrem;
  const int64_t nadd = h.nadd;
  if (!(nadd > 0 && nadd + n - nout < cap)) {  // markers.c:685, 771-774
    if (nadd + n - nout > cap) return MIC_ERR_CAPACITY;
    return MIC_OK;
  }
  // ---- additions ----
  const int64_t nrec = nadd < nout ? nadd : nout;  // new markers that take recycled slots
  const int64_t ncl = ctx->ncells;
  size_t need2 = 0;
  need2 += 3 * (((nadd * sizeof(double)) + 255) / 256) * 256;   // nx ny best_r
  need2 += 14 * (((nadd * sizeof(int)) + 255) / 256) * 256;     // kind tid tslot best_id best_slot next tcell
                                                                // ewrote ecx ecy src ptrA ptrB rslot
  need2 += (((nrec > 0 ? nrec : 1) * sizeof(int) + 255) / 256) * 256;  // clist
  need2 += 2 * ((((ncl + 1) * sizeof(int)) + 255) / 256) * 256;  // cstart cfill
  need2 += 256;                                                 // round flag
  if ((e = ensure_buf(&ctx->dens_add, &ctx->dens_add_bytes, need2))) return e;
  p = (unsigned char *)ctx->dens_add;
  double *nx = carve<double>(p, nadd), *ny = carve<double>(p, nadd), *best_r = carve<double>(p, nadd);
  int *kind = carve<int>(p, nadd), *tid = carve<int>(p, nadd), *tslot = carve<int>(p, nadd);
  int *best_id = carve<int>(p, nadd), *best_slot = carve<int>(p, nadd), *next = carve<int>(p, nadd);
  int *tcell = carve<int>(p, nadd), *ewrote = carve<int>(p, nadd), *ecx = carve<int>(p, nadd);
  int *ecy = carve<int>(p, nadd), *src = carve<int>(p, nadd), *ptrA = carve<int>(p, nadd);
  int *ptrB = carve<int>(p, nadd), *rslot = carve<int>(p, nadd);
  int *clist = carve<int>(p, nrec > 0 ? nrec : 1), *cstart = carve<int>(p, ncl + 1), *cfill = carve<int>(p, ncl + 1);
  int *flags = carve<int>(p, 64);
  // plate_depth(LX) (benchmarkInitialConditions.c:80-91)
  double plate = d->overridingPlateThickness;
  if (fabs(ctx->P.LX - d->rootCenter) < d->rootWidth)
    plate = d->overridingPlateThickness +
            d->rootThickness * pow(cos(M_PI * (ctx->P.LX - d->rootCenter) / d->rootWidth / 2.0), 2.0);
  double wmax = 0.0, hmax = 0.0;
  {
    const double *hx = ctx->h_x + 2;
    const size_t nx4 = (size_t)NX + 4;
    const double *hy = ctx->h_x + 2 * nx4 + 2;
    for (int k = 0; k + 1 < NX; ++k) wmax = fmax(wmax, hx[k + 1] - hx[k]);
    for (int k = 0; k + 1 < NY; ++k) hmax = fmax(hmax, hy[k + 1] - hy[k]);
  }
  {
    MIC_KERNEL(ctx, "k_density_positions");
    k_density_positions<<<grid_for(nq), kBlock, 0, ctx->stream>>>(ctx->P, qadd, nq, s1, plate, (int)nout, n, n,
                                                                   isout, slot_of_id, nx, ny, tid, tslot, kind);
  }
  {
    MIC_KERNEL(ctx, "k_density_nn");
    k_density_nn<<<grid_for(nadd * 32, 128), 128, 0, ctx->stream>>>(ctx->P, ctx->cell_start, c, nx, ny, kind,
                                                                     (int)nadd, wmax, hmax, ctx->P.LX * ctx->P.LY,
                                                                     best_r, best_id, best_slot);
  }
  const int nf = ctx->has_grain ? C_F64_COUNT : C_AOS_F64;
  bool parallel = herr[1] == 0;
  int rounds = 0;
  if (parallel) {
    MIC_CUDA_TRY(cudaMemsetAsync(cstart, 0, sizeof(int) * (ncl + 1), ctx->stream));
    MIC_CUDA_TRY(cudaMemsetAsync(cfill, 0, sizeof(int) * (ncl + 1), ctx->stream));
    if (nrec > 0) {
      {
        MIC_KERNEL(ctx, "k_density_bucket");
        k_density_bucket<<<grid_for(nrec), kBlock, 0, ctx->stream>>>(ctx->P, nx, ny, (int)nrec, tcell, cstart);
      }
      if ((e = mic_scan_exclusive(ctx, cstart, ncl + 1, aux))) return e;
      MIC_KERNEL(ctx, "k_density_scatter");
      k_density_scatter<<<grid_for(nrec), kBlock, 0, ctx->stream>>>(tcell, cstart, (int)nrec, cfill, clist);
    }
    {
      MIC_KERNEL(ctx, "k_density_guess");
      k_density_guess<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(ctx->P, nx, ny, (int)nadd, ewrote, ecx, ecy);
    }
    int jumps = 1;
    while ((1LL << jumps) < nadd + 1) ++jumps;
    constexpr int kMaxRounds = 64;
    int changed = 1;
    while (changed && rounds < kMaxRounds) {
      ++rounds;
      MIC_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int), ctx->stream));
      {
        MIC_KERNEL(ctx, "k_density_decide");
        k_density_decide<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(ctx->P, nx, ny, kind, tid, best_r, best_id,
                                                                     cstart, clist, (int)nadd, wmax, hmax, ewrote,
                                                                     ecx, ecy, src, ptrA);
      }
      int *pin = ptrA, *pout = ptrB;
      for (int k = 0; k < jumps; ++k) {
        MIC_KERNEL(ctx, "k_density_jump");
        k_density_jump<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(pin, pout, (int)nadd);
        int *tmp = pin;
        pin = pout;
        pout = tmp;
      }
      {
        MIC_KERNEL(ctx, "k_density_facts");
        k_density_facts<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(ctx->P, c, nx, ny, kind, tslot, best_slot, src,
                                                                    pin, (int)nadd, ewrote, ecx, ecy, rslot, flags);
      }
      MIC_CUDA_TRY(cudaGetLastError());
      MIC_CUDA_TRY(cudaMemcpyAsync(&changed, flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    parallel = changed == 0;
  }
  ctx->density_rounds = parallel ? rounds : (herr[1] ? -1 : -rounds);
  if (parallel) {
    {
      MIC_KERNEL(ctx, "k_density_build");
      k_density_build<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(ctx->P, ctx->mat, ctx->opt, ctx->creep, c, nf, *d,
                                                                  nx, ny, kind, tid, tslot, (int)nadd, n);
    }
    MIC_KERNEL(ctx, "k_density_copy");
    k_density_copy<<<grid_for(nadd), kBlock, 0, ctx->stream>>>(c, nf, nx, ny, kind, tid, tslot, ewrote, rslot,
                                                               (int)nadd, n);
  } else {  // a slot recycled twice, or no fixed point within the round limit: in order
    MIC_CUDA_TRY(cudaMemsetAsync(heads, 0xFF, sizeof(int) * ctx->ncells, ctx->stream));
    MIC_KERNEL(ctx, "k_density_fill");
    k_density_fill<<<1, 32, 0, ctx->stream>>>(ctx->P, ctx->mat, ctx->opt, ctx->creep, c, nf, *d, nx, ny, kind, tid,
                                              tslot, best_r, best_id, best_slot, (int)nadd, n, wmax, hmax, heads, next);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  ctx->n = n + (nadd > nout ? nadd - nout : 0);
  ctx->rng48 = lcg48_skip(s1, 2ULL * (unsigned long long)nadd);
  ctx->gen++;
  mic_invalidate_sort(ctx);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (n_added) *n_added = nadd;
  return MIC_OK;
}
