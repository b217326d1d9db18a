// mic_context.cu -- context lifecycle, host<->device transfers and status for the C ABI.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include <vector>

#include "mic_internal.cuh"

using namespace mic;

extern "C" int mic_version(void) { return 100; }

extern "C" const char *mic_error_string(int code) {
  switch (code) {
    case MIC_OK: return "ok";
    case MIC_ERR_ARG: return "invalid argument";
    case MIC_ERR_CUDA: return "CUDA runtime error";
    case MIC_ERR_NOMEM: return "out of memory";
    case MIC_ERR_CELL: return "impossible marker cell index";
    case MIC_ERR_NAN: return "NaN strain-rate residual";
    case MIC_ERR_LAW: return "undefined viscosity law";
    case MIC_ERR_BC: return "unsupported boundary condition";
    case MIC_ERR_CAPACITY: return "marker capacity exceeded";
    case MIC_ERR_NO_DEVICE: return "no CUDA device";
    case MIC_ERR_DENSITY: return "marker density control cannot proceed";
    case MIC_ERR_IO: return "checkpoint file could not be read or written";
    case MIC_ERR_SOLVE: return "direct solve failed (zero pivot, or a band too wide)";
    default: return "unknown error";
  }
}

int mic_fail_cuda(mic_ctx *ctx, cudaError_t e) {
  if (ctx) ctx->last_error = (int)e;
  fprintf(stderr, "mic_gb300: CUDA error %d (%s)\n", (int)e, cudaGetErrorString(e));
  return MIC_ERR_CUDA;
}

void mic_invalidate_sort(mic_ctx *ctx) {
  ctx->sorted = 0;
  ctx->geo_valid = 0;
}

// ---- AoS <-> SoA ----------------------------------------------------------------

struct ColPtrs {
  double *f[C_F64_COUNT];
  int *i[C_I32_COUNT];
};

// byte offsets of the f64 columns inside mic_marker, in F64Col order
__constant__ int c_f64_off[C_AOS_F64];
__constant__ int c_i32_off[C_I32_COUNT - 1];  // all but C_ID

static const int h_f64_off[C_AOS_F64] = {
    (int)offsetof(mic_marker, X),     (int)offsetof(mic_marker, Y),     (int)offsetof(mic_marker, VX),
    (int)offsetof(mic_marker, VY),    (int)offsetof(mic_marker, T),     (int)offsetof(mic_marker, Tdot),
    (int)offsetof(mic_marker, s.T11), (int)offsetof(mic_marker, s.T22), (int)offsetof(mic_marker, s.T12),
    (int)offsetof(mic_marker, eta),   (int)offsetof(mic_marker, mu),    (int)offsetof(mic_marker, rho),
    (int)offsetof(mic_marker, rhodot), (int)offsetof(mic_marker, p),    (int)offsetof(mic_marker, e.T11),
    (int)offsetof(mic_marker, e.T22), (int)offsetof(mic_marker, e.T12), (int)offsetof(mic_marker, E.T11),
    (int)offsetof(mic_marker, E.T22), (int)offsetof(mic_marker, E.T12), (int)offsetof(mic_marker, Eii),
    (int)offsetof(mic_marker, wxy),   (int)offsetof(mic_marker, strainRateResidual)};
static const int h_i32_off[C_I32_COUNT - 1] = {(int)offsetof(mic_marker, Mat), (int)offsetof(mic_marker, cellX),
                                               (int)offsetof(mic_marker, cellY), (int)offsetof(mic_marker, cpu),
                                               (int)offsetof(mic_marker, isYielding)};

static_assert(sizeof(mic_marker) == 216, "fvmic2d Marker is 216 bytes");
static_assert(offsetof(mic_marker, cellX) == 184, "fvmic2d Marker layout");

int mic_f64_column_of_offset(int off) {
  for (int c = 0; c < C_AOS_F64; ++c)
    if (h_f64_off[c] == off) return c;
  return -1;
}

__global__ void k_aos_to_soa(const unsigned char *__restrict__ aos, ColPtrs cols, int64_t n) {
  int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const unsigned char *r = aos + m * (int64_t)sizeof(mic_marker);
#pragma unroll
  for (int c = 0; c < C_AOS_F64; ++c) cols.f[c][m] = *reinterpret_cast<const double *>(r + c_f64_off[c]);
#pragma unroll
  for (int c = 0; c < C_I32_COUNT - 1; ++c) cols.i[c][m] = *reinterpret_cast<const int *>(r + c_i32_off[c]);
  cols.i[C_ID][m] = (int)m;
  cols.f[C_GRAIN][m] = kGrainArgDefault;  // default grain size until mic_markers_set_grain_size
}

__global__ void k_soa_to_aos(unsigned char *__restrict__ aos, ColPtrs cols, int64_t n) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int m = cols.i[C_ID][k];
  if (m < 0 || m >= n) return;
  unsigned char *r = aos + (int64_t)m * (int64_t)sizeof(mic_marker);
  memset(r, 0, sizeof(mic_marker));
#pragma unroll
  for (int c = 0; c < C_AOS_F64; ++c) *reinterpret_cast<double *>(r + c_f64_off[c]) = cols.f[c][k];
#pragma unroll
  for (int c = 0; c < C_I32_COUNT - 1; ++c) *reinterpret_cast<int *>(r + c_i32_off[c]) = cols.i[c][k];
}

static ColPtrs cur_cols(mic_ctx *ctx) {
  ColPtrs p;
  for (int c = 0; c < C_F64_COUNT; ++c) p.f[c] = ctx->f64[c];
  for (int c = 0; c < C_I32_COUNT; ++c) p.i[c] = ctx->i32[c];
  return p;
}

// ---- lifecycle --------------------------------------------------------------------

static void prof_free(mic_ctx *ctx);

static void free_ctx(mic_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  prof_free(ctx);
  for (int c = 0; c < C_F64_COUNT; ++c) {
    cudaFree(ctx->f64[c]);
    cudaFree(ctx->f64_alt[c]);
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    cudaFree(ctx->i32[c]);
    cudaFree(ctx->i32_alt[c]);
  }
  for (int f = 0; f < MIC_NF_COUNT; ++f) cudaFree(ctx->nodal[f]);
  for (int f = 0; f < 6; ++f) cudaFree(ctx->node_scr[f]);
  cudaFree(ctx->adv_coef);
  cudaFree(ctx->tickets);
  cudaFree(ctx->grid_buf);
  cudaFree(ctx->bits_buf);
  cudaFree(ctx->spacing_buf);
  cudaFree(ctx->key);
  cudaFree(ctx->key_alt);
  cudaFree(ctx->perm);
  cudaFree(ctx->perm_alt);
  cudaFree(ctx->cell_start);
  cudaFree(ctx->quad_start);
  cudaFree(ctx->part_b);
  cudaFree(ctx->part_c);
  cudaFree(ctx->hist);
  cudaFree(ctx->scan_aux);
  for (int g = 0; g < 4; ++g) cudaFree(ctx->geo[g]);
  cudaFree(ctx->geo_flags);
  cudaFree(ctx->wgt[0]);
  cudaFree(ctx->wgt[1]);
  cudaFree(ctx->scr0);
  cudaFree(ctx->scr1);
  cudaFree(ctx->scr2);
  cudaFree(ctx->red_buf);
  cudaFree(ctx->d_status);
  cudaFree(ctx->d_creep);
  cudaFree(ctx->mlp);
  cudaFree(ctx->train_buf);
  cudaFree(ctx->dens_buf);
  cudaFree(ctx->dens_add);
  cudaFree(ctx->solution);
  cudaFree(ctx->io_buf);
  for (int w = 0; w < 2; ++w) {
    if (ctx->sys[w].lu_exec) cudaGraphExecDestroy(ctx->sys[w].lu_exec);
    cudaFree(ctx->sys[w].cnt);
    cudaFree(ctx->sys[w].col);
    cudaFree(ctx->sys[w].val);
    cudaFree(ctx->sys[w].rhs);
  }
  cudaFree(ctx->sys_scratch);
  cudaFree(ctx->lu_buf);
  if (ctx->lu_side) {
    cudaStreamDestroy(ctx->lu_side);
    cudaEventDestroy(ctx->lu_ev[0]);
    cudaEventDestroy(ctx->lu_ev[1]);
  }
  if (ctx->aux) cudaStreamDestroy(ctx->aux);
  for (int k = 0; k < 2; ++k)
    if (ctx->aux_ev[k]) cudaEventDestroy(ctx->aux_ev[k]);
  cudaFree(ctx->stage_aos);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->owns_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  free(ctx->h_x);
  delete ctx;
}

// The grid tables on the host and the device from the gridlines kept in h_x (x[0..NX-1],
// y[0..NY-1]): cell centres as getCellCenters (gridSpacing.c:150-157); periodic in x, the lines
// and centres beyond the seam as makePeriodic (gridSpacing.c:159-168), x[NX] = LX and NX basic
// cells in x instead of NX - 1.  Order-preserving bit images of the lines and centres (integer
// compares for cell location and the advection's cell walk) and the spacings with their
// reciprocals, every table with 2 ghost entries in front.
static int grid_tables(mic_ctx *ctx, int periodic) {
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const double LX = ctx->P.LX, LY = ctx->P.LY;
  const size_t nx4 = (size_t)NX + 4, ny4 = (size_t)NY + 4;
  double *hx = ctx->h_x + 2, *hxc = ctx->h_x + nx4 + 2, *hy = ctx->h_x + 2 * nx4 + 2,
         *hyc = ctx->h_x + 2 * nx4 + ny4 + 2;
  for (int i = -2; i < 0; ++i) hx[i] = 0.0;
  for (int i = NX; i < NX + 2; ++i) hx[i] = 0.0;
  for (int i = -2; i < NX + 2; ++i) hxc[i] = 0.0;
  for (int j = -2; j < NY + 2; ++j) hyc[j] = 0.0;
  for (int i = 1; i < NX; ++i) hxc[i] = (hx[i - 1] + hx[i]) / 2.0;
  hxc[0] = -hxc[1];
  hxc[NX] = 2.0 * LX - hxc[NX - 1];
  for (int j = 1; j < NY; ++j) hyc[j] = (hy[j - 1] + hy[j]) / 2.0;
  hyc[0] = -hyc[1];
  hyc[NY] = 2.0 * LY - hyc[NY - 1];
  if (periodic) {
    hx[NX] = LX;
    hx[NX + 1] = LX + hx[1];
    hx[-1] = hx[NX - 1] - LX;
    hx[-2] = hx[NX - 2] - LX;
    hxc[NX] = (LX + hx[NX - 1]) / 2.0;
    hxc[NX + 1] = hxc[1] + LX;
    hxc[0] = 0.0 - (LX - hxc[NX]);
    hxc[-1] = 0.0 - (LX - hxc[NX - 1]);
  }
  ctx->h_xc = hxc;
  ctx->h_y = hy;
  ctx->h_yc = hyc;
  ctx->P.xper = periodic ? 1 : 0;
  ctx->P.NCX = periodic ? NX : NX - 1;
  const int NCX = ctx->P.NCX;
  if (cudaMemcpy(ctx->grid_buf, ctx->h_x, sizeof(double) * (2 * nx4 + 2 * ny4), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return MIC_ERR_CUDA;
  // ordered images (a -0.0 line counts as +0.0): lines 0..NCX in x (and -2, -1 beyond the seam),
  // centres 0..NCX+1
  auto ordered = [](double v) {
    long long b;
    memcpy(&b, &v, 8);
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b >= 0 ? b : (long long)(0x8000000000000000ULL) - b;
  };
  std::vector<long long> hb(2 * (nx4 + ny4), 0);
  long long *bx = hb.data() + 2, *by = hb.data() + nx4 + 2, *bxc = hb.data() + nx4 + ny4 + 2,
            *byc = hb.data() + 2 * nx4 + ny4 + 2;
  for (int i = periodic ? -2 : 0; i <= (periodic ? NX + 1 : NX - 1); ++i) bx[i] = ordered(hx[i]);
  for (int j = 0; j < NY; ++j) by[j] = ordered(hy[j]);
  for (int i = periodic ? -1 : 0; i <= (periodic ? NX + 1 : NX); ++i) bxc[i] = ordered(hxc[i]);
  for (int j = 0; j <= NY; ++j) byc[j] = ordered(hyc[j]);
  if (cudaMemcpy(ctx->bits_buf, hb.data(), sizeof(long long) * hb.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return MIC_ERR_CUDA;
  ctx->P.x = ctx->grid_buf + 2;
  ctx->P.xc = ctx->grid_buf + nx4 + 2;
  ctx->P.y = ctx->grid_buf + 2 * nx4 + 2;
  ctx->P.yc = ctx->grid_buf + 2 * nx4 + ny4 + 2;
  ctx->P.xbits = ctx->bits_buf + 2;
  ctx->P.ybits = ctx->bits_buf + nx4 + 2;
  ctx->P.xcbits = ctx->bits_buf + nx4 + ny4 + 2;
  ctx->P.ycbits = ctx->bits_buf + 2 * nx4 + ny4 + 2;
  // spacings h[i] = g[i+1] - g[i] and reciprocals: basic cells 0..NCX-1, centre cells 0..NCX
  // (periodic: also cell -1 beyond the seam), y as before
  std::vector<double> h(4 * nx4 + 4 * ny4, 0.0);
  double *hx_ = h.data() + 2, *ix_ = h.data() + nx4 + 2, *hxc_ = h.data() + 2 * nx4 + 2,
         *ixc_ = h.data() + 3 * nx4 + 2;
  double *hy_ = h.data() + 4 * nx4 + 2, *iy_ = hy_ + ny4, *hyc_ = hy_ + 2 * ny4, *iyc_ = hy_ + 3 * ny4;
  for (int i = periodic ? -1 : 0; i < NCX; ++i) {
    hx_[i] = hx[i + 1] - hx[i];
    ix_[i] = 1.0 / hx_[i];
  }
  for (int i = periodic ? -1 : 0; i <= NCX; ++i) {
    hxc_[i] = hxc[i + 1] - hxc[i];
    ixc_[i] = 1.0 / hxc_[i];
  }
  for (int j = 0; j + 1 < NY; ++j) {
    hy_[j] = hy[j + 1] - hy[j];
    iy_[j] = 1.0 / hy_[j];
  }
  for (int j = 0; j < NY; ++j) {
    hyc_[j] = hyc[j + 1] - hyc[j];
    iyc_[j] = 1.0 / hyc_[j];
  }
  if (cudaMemcpy(ctx->spacing_buf, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return MIC_ERR_CUDA;
  const double *d = ctx->spacing_buf + 2;
  ctx->P.hx = d;
  ctx->P.ix = d + nx4;
  ctx->P.hxc = d + 2 * nx4;
  ctx->P.ixc = d + 3 * nx4;
  ctx->P.hy = d + 4 * nx4;
  ctx->P.iy = d + 4 * nx4 + ny4;
  ctx->P.hyc = d + 4 * nx4 + 2 * ny4;
  ctx->P.iyc = d + 4 * nx4 + 3 * ny4;
  ctx->ncells = NCX * (NY - 1);
  return MIC_OK;
}

#define ALLOC(ptr, bytes)                                                            \
  do {                                                                               \
    if (cudaMalloc((void **)&(ptr), (size_t)(bytes)) != cudaSuccess) {              \
      free_ctx(ctx);                                                                 \
      return MIC_ERR_NOMEM;                                                          \
    }                                                                                \
  } while (0)

extern "C" int mic_create(mic_ctx **out, int device, void *stream, int NX, int NY, double LX, double LY,
                          const double *x, const double *y, int64_t max_markers) {
  if (!out || !x || !y || NX < 3 || NY < 3 || max_markers < 0 || max_markers > (int64_t)0x7FFFFFFF - 4096)
    return MIC_ERR_ARG;
  if ((int64_t)(NX - 1) * (NY - 1) >= (int64_t)0x7FFFFFF0) return MIC_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return MIC_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return MIC_ERR_ARG;
  for (int i = 1; i < NX; ++i)
    if (!(x[i] > x[i - 1])) return MIC_ERR_ARG;
  for (int j = 1; j < NY; ++j)
    if (!(y[j] > y[j - 1])) return MIC_ERR_ARG;
  if (!(x[0] >= 0.0) || !(y[0] >= 0.0)) return MIC_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MIC_ERR_CUDA;
  mic_ctx *ctx = new (std::nothrow) mic_ctx();
  if (!ctx) return MIC_ERR_NOMEM;
  memset((void *)ctx, 0, sizeof(*ctx));
  ctx->device = device;
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return MIC_ERR_CUDA;
    }
    ctx->owns_stream = 1;
  }
  if (cudaStreamCreateWithFlags(&ctx->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->aux_ev[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->aux_ev[1], cudaEventDisableTiming) != cudaSuccess) {
    free_ctx(ctx);
    return MIC_ERR_CUDA;
  }
  // host grid copies with fvmic2d's ghost offset of 2 (the caller's gridlines; the rest of the
  // tables follows from them, periodic or not: grid_tables)
  const size_t nx4 = (size_t)NX + 4, ny4 = (size_t)NY + 4;
  ctx->h_x = (double *)calloc(2 * nx4 + 2 * ny4, sizeof(double));
  if (!ctx->h_x) {
    free_ctx(ctx);
    return MIC_ERR_NOMEM;
  }
  for (int i = 0; i < NX; ++i) ctx->h_x[2 + i] = x[i];
  for (int j = 0; j < NY; ++j) ctx->h_x[2 * nx4 + 2 + j] = y[j];
  ctx->P.NX = NX;
  ctx->P.NY = NY;
  ctx->P.LX = LX;
  ctx->P.LY = LY;
  ALLOC(ctx->grid_buf, sizeof(double) * (2 * nx4 + 2 * ny4));
  ALLOC(ctx->bits_buf, sizeof(long long) * 2 * (nx4 + ny4));
  ALLOC(ctx->spacing_buf, sizeof(double) * (4 * nx4 + 4 * ny4));
  if (grid_tables(ctx, 0) != MIC_OK) {
    free_ctx(ctx);
    return MIC_ERR_CUDA;
  }
  const int64_t cap = max_markers > 0 ? max_markers : 1;
  ctx->cap = cap;
  for (int c = 0; c < C_F64_COUNT; ++c) {  // zeroed: fields no routine has written read as 0
    ALLOC(ctx->f64[c], sizeof(double) * cap);
    ALLOC(ctx->f64_alt[c], sizeof(double) * cap);
    cudaMemset(ctx->f64[c], 0, sizeof(double) * cap);
  }
  for (int c = 0; c < C_I32_COUNT; ++c) {
    ALLOC(ctx->i32[c], sizeof(int) * cap);
    ALLOC(ctx->i32_alt[c], sizeof(int) * cap);
    cudaMemset(ctx->i32[c], 0, sizeof(int) * cap);
  }
  const size_t nn = (size_t)NX * NY;
  for (int f = 0; f < MIC_NF_COUNT; ++f) {
    ALLOC(ctx->nodal[f], sizeof(double) * nn);
    cudaMemset(ctx->nodal[f], 0, sizeof(double) * nn);
  }
  for (int f = 0; f < 6; ++f) ALLOC(ctx->node_scr[f], sizeof(double) * nn);
  // cell arrays sized for the periodic grid's NX x (NY-1) cells (one more column of cells), so
  // that mic_set_bcs can switch periodicity without reallocating
  const size_t max_cells = (size_t)NX * (NY - 1);
  ctx->ncells = ctx->P.NCX * (NY - 1);
  ALLOC(ctx->key, sizeof(int) * cap);
  ALLOC(ctx->key_alt, sizeof(int) * cap);
  ALLOC(ctx->perm, sizeof(int) * cap);
  ALLOC(ctx->perm_alt, sizeof(int) * cap);
  ALLOC(ctx->cell_start, sizeof(int) * (max_cells + 2));
  ALLOC(ctx->quad_start, sizeof(int) * (4 * max_cells + 5));
  ALLOC(ctx->part_b, sizeof(double) * 32 * max_cells);
  ALLOC(ctx->part_c, sizeof(double) * 20 * (size_t)(NX + 1) * NY);  // staggered cells: NX + 1 per row at most
  for (int g = 0; g < 4; ++g) ALLOC(ctx->geo[g], sizeof(double) * cap);
  ALLOC(ctx->geo_flags, sizeof(int) * cap);
#ifndef MIC_EXACT
  ALLOC(ctx->wgt[0], 4 * sizeof(double) * cap);
  ALLOC(ctx->wgt[1], 4 * sizeof(double) * cap);
#endif
  ALLOC(ctx->scr0, sizeof(double) * cap);
  ALLOC(ctx->scr1, sizeof(double) * cap);
  ALLOC(ctx->scr2, sizeof(double) * cap);
  ctx->red_cap = 4096;
  ALLOC(ctx->red_buf, sizeof(double) * ctx->red_cap);
  ALLOC(ctx->d_creep, sizeof(CreepCounters));
  cudaMemset(ctx->d_creep, 0, sizeof(CreepCounters));
  ALLOC(ctx->tickets, sizeof(unsigned int) * BP_COUNT);
  ALLOC(ctx->d_status, sizeof(Status));
  cudaMemset(ctx->d_status, 0, sizeof(Status));
  if (cudaHostAlloc((void **)&ctx->h_status, sizeof(Status), cudaHostAllocDefault) != cudaSuccess) {
    free_ctx(ctx);
    return MIC_ERR_NOMEM;
  }
  memset(ctx->h_status, 0, sizeof(Status));
  cudaMemcpyToSymbol(c_f64_off, h_f64_off, sizeof(h_f64_off));
  cudaMemcpyToSymbol(c_i32_off, h_i32_off, sizeof(h_i32_off));
  for (int b = 0; b < 4; ++b) {
    mic_bcinfo *s = &((mic_bcinfo *)&ctx->bcs)[b];
    for (int k = 0; k < 3; ++k) s->type[k] = 1;
  }
  ctx->mat.nMaterials = 1;
  ctx->rng48 = (1ULL << 16) | 0x330EULL;  // srand48(1), the seed of the reference's main
  ctx->creep.mode = 0;
  ctx->creep.polish_iters = 3;
  ctx->creep.maxit = 60;
  ctx->creep.tol = 2e-14;
  ctx->creep.polish_tol = 1e-7;
  ctx->creep.mlp = nullptr;
  ctx->creep.tc_wait_limit = 1 << 20;  // try_wait rounds on a tensor-core tile (mic_creep_tc.cuh)
  ctx->opt.etamin = 0.0;
  ctx->opt.etamax = 1e300;
  ctx->n = 0;
  ctx->sorted = 0;
  if (cudaDeviceSynchronize() != cudaSuccess || mic_reset_markers(ctx) != MIC_OK) {  // allocateMarkers resets
    free_ctx(ctx);
    return MIC_ERR_CUDA;
  }
  *out = ctx;
  return MIC_OK;
}

extern "C" int mic_destroy(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
  return MIC_OK;
}

extern "C" int mic_set_materials(mic_ctx *ctx, const mic_materials *m) {
  if (!ctx || !m || m->nMaterials < 1 || m->nMaterials > MIC_MAXMAT) return MIC_ERR_ARG;
  ctx->mat = *m;
  ctx->gen++;
  return MIC_OK;
}

extern "C" int mic_set_options(mic_ctx *ctx, const mic_options *o) {
  if (!ctx || !o) return MIC_ERR_ARG;
  ctx->opt = *o;
  ctx->gen++;
  return MIC_OK;
}

// The reference's compile-time JAUMANN switch (markers.c:2147-2164) as a context setting.
extern "C" int mic_set_stress_rotation(mic_ctx *ctx, int rotation) {
  if (!ctx || (rotation != MIC_ROTATION_EXACT && rotation != MIC_ROTATION_JAUMANN)) return MIC_ERR_ARG;
  if (ctx->P.jaumann != (rotation == MIC_ROTATION_JAUMANN)) {
    ctx->P.jaumann = rotation == MIC_ROTATION_JAUMANN;
    ctx->gen++;
  }
  return MIC_OK;
}

extern "C" int mic_get_stress_rotation(mic_ctx *ctx, int *rotation) {
  if (!ctx || !rotation) return MIC_ERR_ARG;
  *rotation = ctx->P.jaumann ? MIC_ROTATION_JAUMANN : MIC_ROTATION_EXACT;
  return MIC_OK;
}

extern "C" int mic_get_bcs(mic_ctx *ctx, mic_bcs *bcs) {
  if (!ctx || !bcs) return MIC_ERR_ARG;
  *bcs = ctx->bcs;
  return MIC_OK;
}

// Boundary values.  A left or right vx type 2 makes the grid periodic in x, as the reference's
// grid generators and nodal DMDAs do (gridGenerator.c:67-68, 97-98; nodalFields.c:11-19): the
// caller's x holds the first NX of NX + 1 lines from 0 to LX, the cells, centres and tables are
// rebuilt, and the markers are binned again.
extern "C" int mic_set_bcs(mic_ctx *ctx, const mic_bcs *b) {
  if (!ctx || !b) return MIC_ERR_ARG;
  const int periodic = b->mechBCLeft.type[0] == 2 || b->mechBCRight.type[0] == 2;
  if (b->mechBCTop.type[0] != 0 && b->mechBCTop.type[0] != 1) return MIC_ERR_BC;
  // the left wall's vy ghost (markers.c:2014-2023) is read only on a non-periodic grid
  if (!periodic && b->mechBCLeft.type[1] != 0 && b->mechBCLeft.type[1] != 1) return MIC_ERR_BC;
  cudaSetDevice(ctx->device);
  if (periodic != ctx->P.xper) {
    // the seam line LX beyond the last line; the sort keys 4 (NX (NY-1)) + 4 fit an int
    if (periodic && (ctx->P.NX < 4 || !(ctx->h_x[2 + ctx->P.NX - 1] < ctx->P.LX) ||
                     4LL * ctx->P.NX * (ctx->P.NY - 1) + 4 >= 0x7FFFFFFFLL))
      return MIC_ERR_ARG;
    cudaError_t ce = cudaStreamSynchronize(ctx->stream);  // the tables are in use by queued work
    if (ce != cudaSuccess) return mic_fail_cuda(ctx, ce);
    const int e = grid_tables(ctx, periodic);
    if (e) return e;
    mic_invalidate_sort(ctx);
  }
  ctx->bcs = *b;
  ctx->gen++;
  return MIC_OK;
}

extern "C" int mic_get_grid_centres(mic_ctx *ctx, double *xc, double *yc) {
  if (!ctx) return MIC_ERR_ARG;
  if (xc)
    for (int i = 0; i <= ctx->P.NX; ++i) xc[i] = ctx->h_xc[i];
  if (yc)
    for (int j = 0; j <= ctx->P.NY; ++j) yc[j] = ctx->h_yc[j];
  return MIC_OK;
}

static int ensure_stage(mic_ctx *ctx, int64_t n) {
  if (ctx->stage_cap >= n) return MIC_OK;
  cudaFree(ctx->stage_aos);
  ctx->stage_aos = nullptr;
  ctx->stage_cap = 0;
  if (cudaMalloc((void **)&ctx->stage_aos, (size_t)n * sizeof(mic_marker)) != cudaSuccess) return MIC_ERR_NOMEM;
  ctx->stage_cap = n;
  return MIC_OK;
}

extern "C" int mic_markers_upload(mic_ctx *ctx, const mic_marker *host, int64_t n) {
  if (!ctx || (n > 0 && !host) || n < 0) return MIC_ERR_ARG;
  if (n > ctx->cap) return MIC_ERR_CAPACITY;
  cudaSetDevice(ctx->device);
  int e = ensure_stage(ctx, n > 0 ? n : 1);
  if (e) return e;
  if (n > 0) {
    MIC_CUDA_TRY(cudaMemcpyAsync(ctx->stage_aos, host, (size_t)n * sizeof(mic_marker), cudaMemcpyHostToDevice,
                                 ctx->stream));
    {
      MIC_KERNEL(ctx, "k_aos_to_soa");
      k_aos_to_soa<<<grid_for(n), kBlock, 0, ctx->stream>>>(ctx->stage_aos, cur_cols(ctx), n);
    }
    MIC_CUDA_TRY(cudaGetLastError());
  }
  ctx->n = n;
  ctx->gen++;
  ctx->has_grain = 0;  // grain column back to its uniform default
  mic_invalidate_sort(ctx);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_markers_download(mic_ctx *ctx, mic_marker *host, int64_t n) {
  if (!ctx || (n > 0 && !host) || n != ctx->n) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n == 0) return MIC_OK;
  int e = ensure_stage(ctx, n);
  if (e) return e;
  {
    MIC_KERNEL(ctx, "k_soa_to_aos");
    k_soa_to_aos<<<grid_for(n), kBlock, 0, ctx->stream>>>(ctx->stage_aos, cur_cols(ctx), n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaMemcpyAsync(host, ctx->stage_aos, (size_t)n * sizeof(mic_marker), cudaMemcpyDeviceToHost,
                               ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_markers_count(mic_ctx *ctx, int64_t *n) {
  if (!ctx || !n) return MIC_ERR_ARG;
  *n = ctx->n;
  return MIC_OK;
}

extern "C" int mic_nodal_upload(mic_ctx *ctx, int f, const double *host) {
  if (!ctx || !host || f < 0 || f >= MIC_NF_COUNT) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaMemcpyAsync(ctx->nodal[f], host, sizeof(double) * (size_t)ctx->P.NX * ctx->P.NY,
                               cudaMemcpyHostToDevice, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_nodal_download(mic_ctx *ctx, int f, double *host) {
  if (!ctx || !host || f < 0 || f >= MIC_NF_COUNT) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaMemcpyAsync(host, ctx->nodal[f], sizeof(double) * (size_t)ctx->P.NX * ctx->P.NY,
                               cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// ---- batched nodal transfers --------------------------------------------------------
//
// Several fields in one call with one synchronization.  When every host buffer is pinned (so the
// device can address it: on Grace-Blackwell over the coherent NVLink-C2C link), one kernel moves
// all of them, element by element, instead of one copy per field; otherwise one asynchronous copy
// per field.
constexpr int kMaxBatch = 32;
struct NodalBatch {
  const double *src[kMaxBatch];
  double *dst[kMaxBatch];
};

__global__ void k_nodal_batch(NodalBatch b, int count, int64_t nn) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nn * count) return;
  const int f = (int)(t / nn);
  const int64_t q = t - (int64_t)f * nn;
  b.dst[f][q] = b.src[f][q];
}

namespace {

// the device address of a host buffer the device can access directly, else null
const void *device_view(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer: not an error for the caller
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return a.devicePointer;
}

int nodal_batch(mic_ctx *ctx, const int *fields, const double *const *host_in, double *const *host_out, int count) {
  if (!ctx || !fields || count < 0 || count > kMaxBatch || (!host_in && !host_out)) return MIC_ERR_ARG;
  for (int k = 0; k < count; ++k) {
    if (fields[k] < 0 || fields[k] >= MIC_NF_COUNT) return MIC_ERR_ARG;
    if (host_in ? !host_in[k] : !host_out[k]) return MIC_ERR_ARG;
  }
  if (count == 0) return MIC_OK;
  cudaSetDevice(ctx->device);
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  NodalBatch b;
  bool direct = true;
  for (int k = 0; k < count && direct; ++k) {
    const void *v = device_view(host_in ? (const void *)host_in[k] : (const void *)host_out[k]);
    if (!v) {
      direct = false;
      break;
    }
    b.src[k] = host_in ? (const double *)v : ctx->nodal[fields[k]];
    b.dst[k] = host_in ? ctx->nodal[fields[k]] : (double *)v;
  }
  if (direct) {
    MIC_KERNEL(ctx, host_in ? "k_nodal_batch_up" : "k_nodal_batch_down");
    k_nodal_batch<<<grid_for(nn * count), kBlock, 0, ctx->stream>>>(b, count, nn);
  } else {
    for (int k = 0; k < count; ++k)
      MIC_CUDA_TRY(host_in ? cudaMemcpyAsync(ctx->nodal[fields[k]], host_in[k], sizeof(double) * nn,
                                             cudaMemcpyHostToDevice, ctx->stream)
                           : cudaMemcpyAsync(host_out[k], ctx->nodal[fields[k]], sizeof(double) * nn,
                                             cudaMemcpyDeviceToHost, ctx->stream));
  }
  MIC_CUDA_TRY(cudaGetLastError());
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

}  // namespace

extern "C" int mic_nodal_upload_many(mic_ctx *ctx, const int *fields, const double *const *host, int count) {
  return nodal_batch(ctx, fields, host, nullptr, count);
}

extern "C" int mic_nodal_download_many(mic_ctx *ctx, const int *fields, double *const *host, int count) {
  return nodal_batch(ctx, fields, nullptr, host, count);
}

extern "C" int mic_nodal_device_ptr(mic_ctx *ctx, int f, double **dev) {
  if (!ctx || !dev || f < 0 || f >= MIC_NF_COUNT) return MIC_ERR_ARG;
  *dev = ctx->nodal[f];
  return MIC_OK;
}

extern "C" int mic_synchronize(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_get_stream(mic_ctx *ctx, void **stream) {
  if (!ctx || !stream) return MIC_ERR_ARG;
  *stream = (void *)ctx->stream;
  return MIC_OK;
}

extern "C" int mic_get_status(mic_ctx *ctx, mic_status *st) {
  if (!ctx || !st) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  st->bad_cell = ctx->h_status->bad_cell;
  st->nan_residual = ctx->h_status->nan_residual;
  st->nan_dsxy = ctx->h_status->nan_dsxy;
  st->bad_law = ctx->h_status->bad_law;
  st->n_out = ctx->h_status->n_out;
  st->is_yielding = ctx->h_status->is_yielding;
  return MIC_OK;
}

extern "C" int mic_debug_sorted_ids(mic_ctx *ctx, int32_t *ids) {
  if (!ctx || !ids) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->n == 0) return MIC_OK;
  MIC_CUDA_TRY(cudaMemcpyAsync(ids, ctx->i32[C_ID], sizeof(int) * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

namespace {
// quotients by the path the kernels use for fractions of a grid spacing: inv = 1 / den
// (correctly rounded), then div_sp(num, den, inv)
__global__ void k_debug_div_sp(const double *num, const double *den, int64_t n, double *q) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  const double d = den[m];
  q[m] = div_sp(num[m], d, 1.0 / d);
}
}  // namespace

// num[k] / den[k] (host arrays) as the kernels divide by a grid spacing (test access)
extern "C" int mic_debug_div_sp(mic_ctx *ctx, const double *num, const double *den, int64_t n, double *quot) {
  if (!ctx || n < 0 || (n > 0 && (!num || !den || !quot))) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n == 0) return MIC_OK;
  double *d = nullptr;
  if (cudaMalloc((void **)&d, sizeof(double) * 3 * (size_t)n) != cudaSuccess) return MIC_ERR_NOMEM;
  cudaError_t ce = cudaMemcpyAsync(d, num, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(d + n, den, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) {
    MIC_KERNEL(ctx, "k_debug_div_sp");
    k_debug_div_sp<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(d, d + n, n, d + 2 * n);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(quot, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
  cudaFree(d);
  return ce == cudaSuccess ? MIC_OK : MIC_ERR_CUDA;
}

extern "C" int mic_debug_cell_start(mic_ctx *ctx, int32_t *cs) {
  if (!ctx || !cs) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaMemcpyAsync(cs, ctx->cell_start, sizeof(int) * ((size_t)ctx->ncells + 2), cudaMemcpyDeviceToHost,
                               ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_host_alloc(void **ptr, int64_t bytes) {
  if (!ptr || bytes <= 0) return MIC_ERR_ARG;
  if (cudaHostAlloc(ptr, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) return MIC_ERR_NOMEM;
  return MIC_OK;
}

extern "C" int mic_host_free(void *ptr) {
  if (!ptr) return MIC_ERR_ARG;
  cudaFreeHost(ptr);
  return MIC_OK;
}

// ---- launch accounting and per-launch timing ------------------------------------------

void mic_prof_begin(mic_ctx *ctx, const char *name, cudaStream_t s) {
  ctx->launches++;
  if (!ctx->prof_on || ctx->prof_n >= ctx->prof_cap) return;
  ctx->prof_name[ctx->prof_n] = name;
  cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n], s);
}

void mic_prof_end(mic_ctx *ctx, cudaStream_t s) {
  if (!ctx->prof_on || ctx->prof_n >= ctx->prof_cap) return;
  cudaEventRecord(ctx->prof_ev[2 * ctx->prof_n + 1], s);
  ctx->prof_n++;
}

static void prof_free(mic_ctx *ctx) {
  for (int k = 0; k < 2 * ctx->prof_cap; ++k) cudaEventDestroy(ctx->prof_ev[k]);
  free(ctx->prof_ev);
  free(ctx->prof_name);
  ctx->prof_ev = nullptr;
  ctx->prof_name = nullptr;
  ctx->prof_cap = ctx->prof_n = 0;
}

// Enables (capacity > 0) or disables (0) per-launch timing; enabling clears the records.
extern "C" int mic_profile_enable(mic_ctx *ctx, int capacity) {
  if (!ctx || capacity < 0) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (capacity == 0) {
    ctx->prof_on = 0;
    return MIC_OK;
  }
  if (capacity != ctx->prof_cap) {
    prof_free(ctx);
    ctx->prof_ev = (cudaEvent_t *)calloc(2 * (size_t)capacity, sizeof(cudaEvent_t));
    ctx->prof_name = (const char **)calloc((size_t)capacity, sizeof(char *));
    if (!ctx->prof_ev || !ctx->prof_name) return MIC_ERR_NOMEM;
    for (int k = 0; k < 2 * capacity; ++k) MIC_CUDA_TRY(cudaEventCreate(&ctx->prof_ev[k]));
    ctx->prof_cap = capacity;
  }
  ctx->prof_n = 0;
  ctx->prof_on = 1;
  return MIC_OK;
}

// Aggregates the recorded launches by kernel name: returns the number of distinct kernels
// and, for k < max, their names (NUL-terminated, 48 bytes each), total ms and launch counts.
extern "C" int mic_profile_read(mic_ctx *ctx, int max, char *names, double *total_ms, int64_t *counts,
                                int *nkernels) {
  if (!ctx || !nkernels) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const char *uniq[128];
  double tot[128];
  int64_t cnt[128];
  int nu = 0;
  for (int r = 0; r < ctx->prof_n; ++r) {
    float ms = 0.f;
    MIC_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->prof_ev[2 * r], ctx->prof_ev[2 * r + 1]));
    int u = 0;
    while (u < nu && strcmp(uniq[u], ctx->prof_name[r]) != 0) ++u;
    if (u == nu) {
      if (nu == 128) continue;
      uniq[nu] = ctx->prof_name[r];
      tot[nu] = 0.0;
      cnt[nu] = 0;
      ++nu;
    }
    tot[u] += ms;
    cnt[u] += 1;
  }
  for (int u = 0; u < nu && u < max; ++u) {
    if (names) {
      strncpy(names + 48 * u, uniq[u], 47);
      names[48 * u + 47] = 0;
    }
    if (total_ms) total_ms[u] = tot[u];
    if (counts) counts[u] = cnt[u];
  }
  *nkernels = nu;
  return MIC_OK;
}

extern "C" int mic_launch_count(mic_ctx *ctx, int64_t *n) {
  if (!ctx || !n) return MIC_ERR_ARG;
  *n = ctx->launches;
  return MIC_OK;
}

// dst[k] = src[id[k]]: a caller-order per-marker array into device (cell-sorted) order
__global__ void k_gather_by_id(const double *__restrict__ src, const int *__restrict__ id, double *__restrict__ dst,
                               int64_t n) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  dst[k] = src[id[k]];
}

int mic_gather_by_id(mic_ctx *ctx, const double *src, double *dst) {
  if (ctx->n == 0) return MIC_OK;
  {
    MIC_KERNEL(ctx, "k_gather_by_id");
    k_gather_by_id<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(src, ctx->i32[C_ID], dst, ctx->n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

// ---- marker lifecycle: resetMarkers, distributeMarkersUniformInDomain, field fills ----------

// resetMarker (markers.c:255-330) on every slot of the capacity; mu, cellX, cellY, cpu and the
// strain-rate residual are left as they are, as in the reference
__global__ void k_reset_markers(ColPtrs c, int64_t cap) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= cap) return;
  c.f[C_X][m] = -1.0;
  c.f[C_Y][m] = -1.0;
  const int zero[] = {C_VX, C_VY, C_T, C_TDOT, C_SXX, C_SYY, C_SXY, C_ETA, C_RHO, C_RHODOT, C_P,
                      C_EXX, C_EYY, C_EXY, C_EXX_TOT, C_EYY_TOT, C_EXY_TOT, C_EII, C_WXY};
#pragma unroll
  for (int q = 0; q < (int)(sizeof(zero) / sizeof(zero[0])); ++q) c.f[zero[q]][m] = 0.0;
  c.f[C_GRAIN][m] = kGrainArgDefault;
  c.i[C_MAT][m] = -1;
  c.i[C_ISYIELD][m] = 0;
}

// The single-rank PETSc random stream of distributeMarkersUniformInDomain: 48-bit state
// X <- (0x5DEECE66D X + 11) mod 2^48 from (seed << 16) | 0x330E, value u = X / 2^48 after each
// step.  k steps at once: the affine map x -> A x + C composed k times (binary powers).
__device__ __forceinline__ unsigned long long lcg48_after(unsigned long long x0, unsigned long long k) {
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

// PetscRandomGetValue on [lo, hi) after `calls` earlier values; the reference's expression
// order, without contraction
__device__ __forceinline__ double stream_value(unsigned long long x0, unsigned long long calls, double lo,
                                               double hi) {
  const double u = (double)lcg48_after(x0, calls + 1) * (1.0 / 281474976710656.0);
  return __dadd_rn(lo, __dmul_rn(__dsub_rn(hi, lo), u));
}

// distributeMarkersUniformInDomain (markers.c:342-400): marker idx = k * nyl + l at
// x0 + mdx (0.5 + k) + U(-mdx/4, mdx/4), y0 + mdy (0.5 + l) + U(-mdy/4, mdy/4), two values per
// marker from the stream in marker order
__global__ void k_distribute(ColPtrs c, int64_t n, int nyl, double x0, double y0, double mdx, double mdy,
                             unsigned long long state0) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int64_t k = idx / nyl, l = idx % nyl;
  const double tx = stream_value(state0, 2ULL * (unsigned long long)idx, -mdx / 4.0, mdx / 4.0);
  const double ty = stream_value(state0, 2ULL * (unsigned long long)idx + 1ULL, -mdy / 4.0, mdy / 4.0);
  c.f[C_X][idx] = __dadd_rn(__dadd_rn(x0, __dmul_rn(mdx, 0.5 + (double)k)), tx);
  c.f[C_Y][idx] = __dadd_rn(__dadd_rn(y0, __dmul_rn(mdy, 0.5 + (double)l)), ty);
  c.i[C_ID][idx] = (int)idx;
}

__global__ void k_fill_f64(double *col, double v, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < n) col[m] = v;
}

__global__ void k_fill_i32(int *col, int v, int64_t n) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m < n) col[m] = v;
}

// resetMarker (markers.c:255-330) on a host array: the same values k_reset_markers gives the
// device columns, for host code that owns a marker array before any context exists
// (allocateMarkers resets its fresh array)
extern "C" int mic_markers_reset_host(mic_marker *m, int64_t n) {
  if (n < 0 || (n > 0 && !m)) return MIC_ERR_ARG;
  for (int64_t k = 0; k < n; ++k) {
    mic_marker &r = m[k];
    r.X = -1.0;
    r.Y = -1.0;
    r.VX = r.VY = 0.0;
    r.T = r.Tdot = 0.0;
    r.s.T11 = r.s.T22 = r.s.T12 = 0.0;
    r.eta = 0.0;
    r.rho = r.rhodot = 0.0;
    r.p = 0.0;
    r.e.T11 = r.e.T22 = r.e.T12 = 0.0;
    r.E.T11 = r.E.T22 = r.E.T12 = 0.0;
    r.Eii = 0.0;
    r.wxy = 0.0;
    r.Mat = -1;
    r.isYielding = 0;
  }
  return MIC_OK;
}

extern "C" int mic_reset_markers(mic_ctx *ctx) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->cap > 0) {
    MIC_KERNEL(ctx, "k_reset_markers");
    k_reset_markers<<<grid_for(ctx->cap), kBlock, 0, ctx->stream>>>(cur_cols(ctx), ctx->cap);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  ctx->has_grain = 0;
  ctx->gen++;
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_distribute_markers_uniform_in_domain(mic_ctx *ctx, int NMX, int NMY, unsigned long seed,
                                                        int64_t *n_placed) {
  if (!ctx || NMX < 1 || NMY < 1) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int NX = ctx->P.NX, NY = ctx->P.NY;
  const double *hx = ctx->h_x + 2;
  const size_t nx4 = (size_t)NX + 4;
  const double *hy = ctx->h_x + 2 * nx4 + 2;
  // markers.c:367-375, one rank owning the whole grid
  const double mdx = ctx->P.LX / (NMX * (NX - 1));
  const double mdy = ctx->P.LY / (NMY * (NY - 1));
  const int nxl = (int)((hx[NX - 1] - hx[0]) / mdx);
  const int nyl = (int)((hy[NY - 1] - hy[0]) / mdy);
  const int64_t n = (int64_t)(nxl > 0 ? nxl : 0) * (int64_t)(nyl > 0 ? nyl : 0);
  if (n > ctx->cap) return MIC_ERR_CAPACITY;
  int e;
  // the reference writes X, Y into array slots 0..n-1 and leaves every other field as it was
  if (ctx->n > 0 && (e = mic_restore_caller_order(ctx))) return e;
  if (n > 0) {
    const unsigned long long state0 = ((unsigned long long)(seed & 0xFFFFFFFFUL) << 16) | 0x330EULL;
    MIC_KERNEL(ctx, "k_distribute");
    k_distribute<<<grid_for(n), kBlock, 0, ctx->stream>>>(cur_cols(ctx), n, nyl, hx[0], hy[0], mdx, mdy, state0);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  ctx->n = n;
  ctx->gen++;
  mic_invalidate_sort(ctx);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (n_placed) *n_placed = n;
  return MIC_OK;
}

extern "C" int mic_markers_fill(mic_ctx *ctx, int field_offset, double value) {
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  const int fc = mic_f64_column_of_offset(field_offset);
  int ic = -1;
  for (int c = 0; c < C_I32_COUNT - 1; ++c)
    if (h_i32_off[c] == field_offset) ic = c;
  if (fc < 0 && ic < 0) return MIC_ERR_ARG;
  if (ctx->n > 0) {
    MIC_KERNEL(ctx, "k_fill");
    if (fc >= 0)
      k_fill_f64<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->f64[fc], value, ctx->n);
    else
      k_fill_i32<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->i32[ic], (int)value, ctx->n);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  if (ic == C_CELLX || ic == C_CELLY || fc == C_X || fc == C_Y) mic_invalidate_sort(ctx);
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

extern "C" int mic_marker_count(mic_ctx *ctx, int64_t *n) {
  if (!ctx || !n) return MIC_ERR_ARG;
  *n = ctx->n;
  return MIC_OK;
}
