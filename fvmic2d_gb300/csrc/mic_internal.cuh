// mic_internal.cuh -- device context and helpers shared by the GB300 marker-in-cell kernels.
//
// Markers live on the device as structure-of-arrays columns, physically ordered by
// cell after every binning (stable counting sort by linear cell id, out-of-domain
// markers last).  Column `id` keeps each marker's index in the caller's array so
// that host transfers restore the caller's order.
//
// Nodal fields are NX*NY doubles, x fastest, one device array per field id of
// include/mic_types.h.  Grid arrays x, y, xc, yc keep fvmic2d's two ghost entries
// on each side (gridGenerator.c:123-130); the device copies point at entry 0.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mic_gb300.h"
#include "mic_types.h"

namespace mic {

// double-valued marker columns, in mic_marker field order
enum F64Col {
  C_X = 0, C_Y, C_VX, C_VY, C_T, C_TDOT, C_SXX, C_SYY, C_SXY, C_ETA, C_MU, C_RHO, C_RHODOT, C_P,
  C_EXX, C_EYY, C_EXY, C_EXX_TOT, C_EYY_TOT, C_EXY_TOT, C_EII, C_WXY, C_SRR,
  C_AOS_F64,              // columns above mirror mic_marker fields; those below are device-only
  C_GRAIN = C_AOS_F64,    // grain argument of the composite creep law (law 7): grain_arg(d)
  C_F64_COUNT
};
// grain argument of the default grain size d = 1 mm (until mic_markers_set_grain_size): d itself
// in the FMA-free parity build, d^-0.2 = 10^0.6 in the product build (mic_creep.cuh, grain_arg)
#ifdef MIC_EXACT
constexpr double kGrainArgDefault = 1e-3;
#else
constexpr double kGrainArgDefault = 3.9810717055349727;
#endif
// int-valued marker columns
enum I32Col { C_MAT = 0, C_CELLX, C_CELLY, C_CPU, C_ISYIELD, C_ID, C_I32_COUNT };

// device status word (counts of events the reference aborts or prints on)
struct Status {
  unsigned long long bad_cell;      // impossible cell index (markers.c:74-77)
  unsigned long long nan_residual;  // NaN strain-rate residual (updateMarkerStrainPressure.c:302-306)
  unsigned long long nan_dsxy;      // NaN interpolated dsxy (updateMarkerStress.c:136-142)
  unsigned long long bad_law;       // unknown viscosity law (viscosity.c:60-62)
  unsigned long long n_out;         // out-of-domain markers after the last binning
  int is_yielding;                  // any marker yielded in the last checkPlasticYielding
  int pad;
};

// Composite creep (law 7) settings and per-pass counters
struct CreepConfig {
  int mode;             // 0: exact Newton; 1: surrogate guess + polish + exact fallback
  int polish_iters;     // Newton steps after the surrogate guess
  int maxit;            // iteration cap of the exact solve
  double tol;           // exact solve: |rate/edot - 1| <= tol
  double polish_tol;    // surrogate path: residual above this after polishing -> exact fallback
  const float *mlp;     // surrogate network parameters (device), see mic_creep.cu
  int tc_wait_limit;    // try_wait rounds on a tensor-core tile's completion before giving up
};

struct CreepCounters {
  unsigned long long markers, iterations, fallbacks;
  unsigned long long max_res_bits;  // bits of the largest |rate/edot - 1| (non-negative double)
  unsigned long long tc_timeouts;   // tensor-core tiles whose completion wait ran out
  unsigned long long tc_drain_timeouts;  // blocks whose final drain ran out before TMEM was freed
};

struct Params {  // everything a kernel needs besides the marker columns; passed by value
  int NX, NY;
  int NCX;   // basic cells in x: NX - 1, or NX on a grid periodic in x (line NX is line 0's image)
  int xper;  // periodic in x: node column NX is column 0, NX + 1 is 1, -1 is NX - 1
  int jaumann;  // stress rotation of the advection: 1 the first-order Jaumann update (markers.c:2147-2156,
                // the reference built with -DJAUMANN), 0 the exact rotation (2158-2164)
  double LX, LY;
  const double *x, *y, *xc, *yc;  // point at index 0 (ghost entries at -2, -1 exist)
  const long long *xbits, *ybits; // bit patterns of x[0..NX-1], y[0..NY-1] for integer compares
  const long long *xcbits, *ycbits;  // ordered_bits of xc[0..NX], yc[0..NY] (xc[0], yc[0] < 0)
  // cell spacings h[i] = g[i+1] - g[i] (the reference's own differences) and their correctly
  // rounded reciprocals, for basic lines (i in [0, N-2]) and cell centres (i in [0, N-1])
  const double *hx, *ix, *hy, *iy, *hxc, *ixc, *hyc, *iyc;
};

}  // namespace mic

// one assembled linear system: rows of at most `width` (column, value) entries, the right-hand
// side, and the banded factorisation state
struct mic_system_store {
  int64_t n;
  int width;
  int *cnt, *col;
  double *val, *rhs;
  double Kbond, Kcont;
  int factored;
  int kl, ku;       // band widths of the last factorisation
  int zero_pivot;   // first zero pivot of the last factorisation (-1: none)
  // the factorisation's launches captured as a graph, valid for this buffer, size, band, panel
  cudaGraphExec_t lu_exec;
  const void *lu_key_buf;
  int64_t lu_key_n;
  int lu_key_kl, lu_key_ku, lu_key_nb;
  long long lu_nodes;
};

struct mic_ctx {
  int device;
  cudaStream_t stream;
  int owns_stream;
  mic::Params P;
  double *grid_buf;  // device: x, xc, y, yc with ghosts
  double *spacing_buf;  // device: hx, ix, hy, iy, hxc, ixc, hyc, iyc
  long long *bits_buf;
  double *h_x, *h_y, *h_xc, *h_yc;  // host copies (with ghosts)
  mic_materials mat;
  mic_options opt;
  mic_bcs bcs;
  mic::CreepConfig creep;
  mic::CreepCounters *d_creep;  // device counters of the last rheology pass
  float *mlp;                   // device surrogate parameters
  unsigned long long mlp_key;   // content key of *mlp (0: not known)
  float *train_buf;             // training scratch (grown on demand)
  int64_t train_cap;
  int64_t n, cap;
  int has_grain;  // per-marker grain sizes were set: the grain column moves with the sorts
  long long gen;  // bumped by every setter that changes what a step launches (captured graphs)
  unsigned long long rng48;  // drand48 stream of marker density control (48-bit state)
  int density_rounds;        // rounds of the last parallel fill; negative: the in-order fill ran
  void *dens_buf, *dens_add;  // density-control scratch (grown on demand)
  double *solution;           // Stokes solution (3 NX NY, dof-interleaved) for retrieveSolutions
  void *io_buf;               // checkpoint packing scratch (grown on demand)
  mic_system_store sys[2];    // assembled systems: 0 Stokes (vep_system.c), 1 thermal
  void *sys_scratch;          // assembly scratch: geometry tables, scaled viscosities
  size_t sys_scratch_bytes;
  void *lu_buf;               // banded factorisation storage (grown on demand)
  size_t lu_bytes;
  cudaStream_t lu_side;       // second stream of the factorisation: the far part of each update
  cudaEvent_t lu_ev[2];       // its two hand-offs (trsm done, far update done)
  cudaStream_t aux;           // second stream of a projection: its cell-centre partial sums run
  cudaEvent_t aux_ev[2];      // beside the basic-cell ones (fork, join)
  size_t io_bytes;
  size_t dens_bytes, dens_add_bytes;
  double *f64[mic::C_F64_COUNT];
  int *i32[mic::C_I32_COUNT];
  double *f64_alt[mic::C_F64_COUNT];
  int *i32_alt[mic::C_I32_COUNT];
  double *nodal[MIC_NF_COUNT];
  // binning / sort scratch
  int ncells;
  int *key, *key_alt, *perm, *perm_alt;
  int *cell_start;     // ncells + 2 entries
  int *quad_start;     // 4*ncells + 5 entries: runs of each (cell, quadrant)
  double *part_b, *part_c;  // per-cell corner partial sums of the projections (product build)
  int *hist;           // radix histograms (digit-major per tile)
  int hist_cap;
  int *scan_aux;
  int sorted;          // columns are in cell order for the current positions
  // per-marker projection geometry for the current positions and order (see mic_project.cu)
  double *geo[4];      // mdx0, mdy0 (basic cell), mdx1, mdy1 (cell-centre stagger -1,-1)
  int *geo_flags;      // bit0 qx, bit1 qy, bit2 mdx0>=.5, bit3 mdy0>=.5, bit4 mdx1>=.5, bit5 mdy1>=.5
  double *wgt[2];      // bilinear corner weights (product build), 4 per marker in corner order
                       // 00, 10, 01, 11: [0] of the basic cell, [1] of the cell-centre cell
  int geo_valid;
  // per-marker scratch
  double *scr0, *scr1, *scr2;
  double *node_scr[6];  // nodal scratch (NX*NY each)
  void *adv_coef;       // per-cell bilinear coefficients of vx, vy, wxy for the advection (product build)
  unsigned int *tickets;  // per marker pass: the tile counter of a dynamic walk (mic_batch_launch's walk 2)
  double *red_buf;     // reduction partials
  int red_cap;
  mic::Status *d_status;
  mic::Status *h_status;  // pinned mirror
  unsigned char *stage_aos;  // device staging for AoS transfers
  int64_t stage_cap;
  double residuals[100];
  int last_error;
  // launch accounting and optional per-launch CUDA-event timing
  long long launches;
  int tune_bs[16];  // launch block size per tuned kernel (TuneId); 0 = kBlock
  int prof_on;
  int prof_n, prof_cap;
  const char **prof_name;
  cudaEvent_t *prof_ev;  // 2 per record
};

void mic_prof_begin(mic_ctx *ctx, const char *name, cudaStream_t s);
void mic_prof_end(mic_ctx *ctx, cudaStream_t s);

namespace mic {
struct ProfScope {  // brackets one kernel launch: counts it and, when enabled, times it
  mic_ctx *c;
  cudaStream_t s;
  ProfScope(mic_ctx *ctx, const char *name, cudaStream_t st) : c(ctx), s(st) { mic_prof_begin(ctx, name, st); }
  ~ProfScope() { mic_prof_end(c, s); }
};
}  // namespace mic
#define MIC_KERNEL(ctx, name) mic::ProfScope _mic_prof_scope(ctx, name, (ctx)->stream)
#define MIC_KERNEL_ON(ctx, name, st) mic::ProfScope _mic_prof_scope(ctx, name, st)

// ---- helpers -------------------------------------------------------------------------

#define MIC_CUDA_TRY(expr)                                  \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return mic_fail_cuda(ctx, _e);   \
  } while (0)

int mic_fail_cuda(mic_ctx *ctx, cudaError_t e);
int mic_ensure_sorted(mic_ctx *ctx);  // bins + sorts if positions changed since the last sort
// ARITHMETIC projection of a marker value column (binned order) to basic nodes (stag 0) or cell
// centres (stag -1), divided by the weights
int mic_project_scalar(mic_ctx *ctx, const double *v, int stag, double *out, cudaStream_t s = nullptr);
void mic_invalidate_sort(mic_ctx *ctx);
int mic_bin_and_sort(mic_ctx *ctx, int64_t *n_out);
int mic_ensure_geometry(mic_ctx *ctx);  // sorted columns + projection geometry
// projectMarkersNodesAll2 again after a full pass on unchanged positions, densities, temperatures
// and materials (only viscosities and stresses changed): the product build re-forms only those
int mic_project_all2_viscous(mic_ctx *ctx);
// the step's first projectMarkersNodesAll2 when mic_project_all2_viscous follows before any of
// its viscosity or stress fields is read: the product build forms only rho, k, T, Cp (and the
// weights the viscous pass divides by), on stream s; the exact build projects everything
int mic_project_all2_first(mic_ctx *ctx, cudaStream_t s);
// copies of a context's marker columns and nodal fields, put back by mic_state_restore
int mic_state_save(mic_ctx *ctx, void **handle);
int mic_state_restore(mic_ctx *ctx, void *handle);
void mic_state_free(void *handle);
int mic_f64_column_of_offset(int byte_offset);
// exclusive prefix sum in place on the context stream, and the scratch it needs (mic_bin_sort.cu)
int mic_scan_exclusive(mic_ctx *ctx, int *data, int64_t len, int *aux);
int64_t mic_scan_aux_ints(int64_t len);
// columns [0, n) back to caller order, slots from n on kept (mic_bin_sort.cu)
int mic_restore_caller_order(mic_ctx *ctx);
// scatter a caller-order per-marker array into device (column) order through the id column
int mic_gather_by_id(mic_ctx *ctx, const double *src, double *dst);
// persistent block count of the tensor-core creep kernels for n markers (mic_creep_tc.cu)
int mic_creep_tc_blocks(mic_ctx *ctx, int64_t n);
// network outputs for device features (n x 4) on the tensor cores (mic_creep_tc.cu)
int mic_mlp_infer_tc_launch(mic_ctx *ctx, const float *feat, int64_t n, float *y);
// tensor-core creep surrogate over a device batch (mic_creep_tc.cu)
int mic_creep_surrogate_tc_launch(mic_ctx *ctx, const double *edot, const double *T, const double *d,
                                  const double *P, int64_t n, double *s, int *it, double *res, int *fb);

// ---- one step in segments, and marker passes batched over many contexts (mic_marker_passes.cu)

namespace mic {
// The marker passes of a step a batch gathers: one batched kernel each.  The yield pass has one
// per creep variant (no law-7 material, exact solve, FP32 surrogate, tensor-core surrogate).
enum BatchPass {
  BP_RHO = 0,
  BP_YIELD_PLAIN,
  BP_YIELD_EXACT,
  BP_YIELD_FP32,
  BP_YIELD_TC,
  BP_STRAIN,
  BP_SUBGRID,
  BP_STRESS,
  BP_SUBT,
  BP_SUBT_APPLY,
  BP_ADVECT,
  BP_COUNT
};
// How a batched kernel walks its work table: tiles of `mult` x block-size markers, each inside
// one member; one block per tile, or a persistent grid (SMs x resident blocks) whose blocks take
// tiles round-robin or as one contiguous run each (chunked).
struct BatchShape {
  int mult, persistent, chunked;
};
constexpr int kStepSegments = 10;
}  // namespace mic

struct mic_batch;  // the marker-pass jobs of one segment, gathered over the members
mic_batch *mic_batch_new();
void mic_batch_free(mic_batch *b);
bool mic_batch_empty(const mic_batch *b);
void mic_batch_clear(mic_batch *b);
// bytes of work table one ensemble step of n_members contexts needs at most
size_t mic_batch_table_bound(int n_members);
// Segment seg (0 .. kStepSegments-1) of one step: the context's own launches up to and including
// one marker pass, on its stream.  Segments 0 .. kStepSegments-1 in order are mic_step without its
// residual read.  With b, the segment's marker pass joins the batch instead of being launched.
// wz_known: the advection may take the marker vorticity of this step's strain-rate pass.
int mic_step_segment(mic_ctx *ctx, int seg, double dt_disp, double dt_thermal, int subgrid_stress, int wz_known,
                     mic_batch *b);
// Launch every pass the batch holds on stream s, each as one kernel over its jobs (in the order
// they were added) with its shape; the jobs and the tile table are written into host_table at
// *off (advanced; cap bytes in all) and read by the kernels from the same offset of dev_table.
// copy: enqueue the host-to-device copy of the written bytes on s first (else the caller copies
// the table before the launches run).  *launches counts the kernels.  Empties the batch.
int mic_batch_launch(mic_batch *b, const mic::BatchShape *shape, unsigned char *host_table, unsigned char *dev_table,
                     size_t *off, size_t cap, int copy, cudaStream_t s, long long *launches);

namespace mic {

constexpr int kBlock = 256;

// Marker-parallel kernels whose block size mic_autotune picks (each uses at most 96 registers,
// so every candidate up to 512 threads fits an SM's register file).
enum TuneId {
  TU_ADVECT = 0,
  TU_STRAIN,
  TU_YIELD,
  TU_SUBGRID_STRESS,
  TU_UPDATE_STRESS,
  TU_SUBGRID_T,
  TU_SUBGRID_T_APPLY,
  TU_REORDER,
  TU_FIND_CELLS,
  TU_UPDATE_RHO,
  TU_COUNT
};

inline unsigned grid_for(int64_t n, int block = kBlock);
inline int tuned_block(const mic_ctx *ctx, int id) {
  const int b = ctx->tune_bs[id];
  return b > 0 ? b : kBlock;
}
inline unsigned grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  return (unsigned)(g < 1 ? 1 : g);
}
// streaming multiprocessors of the context's device (cached per device ordinal)
inline int sm_count(const mic_ctx *ctx) {
  static int cache[64];
  const int d = ctx->device;
  if (d >= 0 && d < 64 && cache[d] > 0) return cache[d];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || n < 1) n = 1;
  if (d >= 0 && d < 64) cache[d] = n;
  return n;
}

// Bit pattern of a non-negative double, canonicalising -0.0 to +0.0, so that for
// non-negative finite values a >= b  <=>  bits(a) >= bits(b) as signed integers.
// Bilinear weights (1-mdx)(1-mdy), mdx(1-mdy), (1-mdx)mdy, mdx mdy, formed as the reference's
// interpolations form them.
struct W4 {
  double w00, w10, w01, w11;
};
__device__ __forceinline__ W4 make_w4(double mdx, double mdy) {
  const double a = 1.0 - mdx, b = 1.0 - mdy;
  return W4{a * b, mdx * b, a * mdy, mdx * mdy};
}
__device__ __forceinline__ W4 load_w4(const double *__restrict__ w, int64_t m) {
  const double2 lo = __ldg(reinterpret_cast<const double2 *>(w + 4 * m));
  const double2 hi = __ldg(reinterpret_cast<const double2 *>(w + 4 * m) + 1);
  return W4{lo.x, lo.y, hi.x, hi.y};
}
// weight of corner k = ox + 2 oy (selects, no FP64 work)
__device__ __forceinline__ double w4_at(const W4 &w, int k) {
  return (k & 2) ? ((k & 1) ? w.w11 : w.w01) : ((k & 1) ? w.w10 : w.w00);
}
__device__ __forceinline__ void store_w4(double *w, int64_t m, const W4 &v) {
  reinterpret_cast<double2 *>(w + 4 * m)[0] = make_double2(v.w00, v.w10);
  reinterpret_cast<double2 *>(w + 4 * m)[1] = make_double2(v.w01, v.w11);
}

// The bit pattern of v through an opaque 64-bit move.  The integer tests and conversions built on
// it stay integer instructions: on a double computed in registers the compiler otherwise may turn
// a test of its bits back into FP64 instructions (measured: an FP64 add per test), which take
// slots of the FP64 pipe these tests exist to spare.
__device__ __forceinline__ long long dbits(double v) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
  return b;
}

__device__ __forceinline__ long long nonneg_bits(double v) {
  long long b = dbits(v);
  return (b == (long long)0x8000000000000000ULL) ? 0LL : b;
}

// Order-preserving map of any non-NaN double to a signed integer key.
__device__ __forceinline__ long long ordered_bits(double v) {
  long long b = dbits(v);
  return b >= 0 ? b : (long long)(0x8000000000000000ULL) - b;
}

// true for a NaN bit pattern (integer test: no FP64 instruction)
__device__ __forceinline__ bool nan_bits(long long b) {
  return (b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL;
}

// Conversions and compares by bit pattern.  On GB300 every conversion to or from FP64 and every
// FP64 compare or min/max takes a slot of the FP64 pipe (2 per SM per clock), the bound of the
// FP64-heavy marker passes; these forms use integer instructions only.

// a < c for a positive finite constant c and any a; false for NaN (as the FP64 compare)
__device__ __forceinline__ bool lt_pos(double a, double c) {
  const long long b = dbits(a);
  return b < dbits(c) && !nan_bits(b);
}
// a > 0, false for zero of either sign and for NaN (as the FP64 compare)
__device__ __forceinline__ bool gt_zero(double a) {
  const long long b = dbits(a);
  return b > 0 && b <= 0x7FF0000000000000LL;
}
// |a| <= c for c >= 0 (not NaN); false for a NaN a
__device__ __forceinline__ bool abs_le(double a, double c) {
  return (dbits(a) & 0x7FFFFFFFFFFFFFFFLL) <= dbits(c);
}

// FP32 copy of v scaled by 2^-k, from its bit pattern: the exponent re-biased and the mantissa
// truncated to 23 bits (relative error below 2^-23, against 2^-24 for a rounding conversion);
// signed zero below FP32's normal range, infinity above it, NaN for NaN.
__device__ __forceinline__ float f32_trunc(double v, int k = 0) {
  const long long b = dbits(v);
  const unsigned hi = (unsigned)((unsigned long long)b >> 32);
  const unsigned s = hi & 0x80000000u;
  const int eb = (int)((hi >> 20) & 0x7FFu);
  const int e = eb - 896 - k;
  unsigned r = s | ((unsigned)e << 23) | ((unsigned)((unsigned long long)b >> 29) & 0x7FFFFFu);
  if (e <= 0 || eb == 0) r = s;
  if (e >= 255 || eb == 0x7FF) r = s | (nan_bits(b) ? 0x7FC00000u : 0x7F800000u);
  return __uint_as_float(r);
}
// binary exponent of a positive normal double (floor(log2 v))
__device__ __forceinline__ int exp2_of(double v) {
  return (int)(((unsigned long long)dbits(v) >> 52) & 0x7FF) - 1023;
}
// exact FP64 value of f from its bit pattern: normal floats, infinities and NaN; zero and the FP32
// subnormals (below 1.2e-38) give signed zero
__device__ __forceinline__ double f64_of(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned long long m = (unsigned long long)(u & 0x7FFFFFu) << 29;
  unsigned long long r = s | ((unsigned long long)(e + 896u) << 52) | m;
  if (e == 0) r = s;
  if (e == 255) r = s | 0x7FF0000000000000ULL | m;
  return __longlong_as_double((long long)r);
}

// a / 6 from the correctly rounded reciprocal, corrected by one residual step (Markstein)
__device__ __forceinline__ double div6(double a) {
#ifdef MIC_EXACT
  return a / 6;
#else
  const double inv6 = 0.16666666666666666;
  const double q = a * inv6;
  return fma(fma(-q, 6.0, a), inv6, q);
#endif
}

// num / den for a grid-spacing divisor den whose correctly rounded reciprocal is inv.  The
// FMA-free parity build divides.  The product build multiplies by the reciprocal and corrects
// the quotient with one residual step (Markstein): q = num*inv, e = num - q*den (exact with
// FMA), q + e*inv -- the correctly rounded quotient, for a third of a division's FP64 work.
__device__ __forceinline__ double div_sp(double num, double den, double inv) {
#ifdef MIC_EXACT
  (void)inv;
  return num / den;
#else
  const double q = num * inv;
  const double e = fma(-q, den, num);
  return fma(e, inv, q);
#endif
}

// Running bilinear sum in the order 00, 01, 10, 11 of updateMarkerStrainPressure.c:152-158,
// subgridStressChanges.c:97-102 and updateMarkerStress.c:84-93.
// The same running sum with the weights given.
// Node column i + 1 wraps to 0 at NX: only on a grid periodic in x does an interpolation cell
// reach column NX (the seam's image of column 0); elsewhere i + 1 <= NX - 1.
__device__ __forceinline__ int next_col(int i, int NX) { return (i + 1 == NX) ? 0 : i + 1; }
// node column of a periodic local index in [-NX, 2 NX)
__device__ __forceinline__ int wrap_col(int i, int NX) { return i < 0 ? i + NX : (i >= NX ? i - NX : i); }

__device__ __forceinline__ double interp_w(const double *__restrict__ f, int NX, int i, int j, const W4 &w) {
  const size_t r0 = (size_t)j * NX, r1 = r0 + NX;
  const int i1 = next_col(i, NX);
  double s = w.w00 * __ldg(f + r0 + i);
  s = fma(w.w01, __ldg(f + r1 + i), s);
  s = fma(w.w10, __ldg(f + r0 + i1), s);
  s = fma(w.w11, __ldg(f + r1 + i1), s);
  return s;
}

__device__ __forceinline__ double interp_run(const double *__restrict__ f, int NX, int i, int j, double mdx,
                                             double mdy) {
  const size_t r0 = (size_t)j * NX, r1 = r0 + NX;
  const int i1 = next_col(i, NX);
  double s = 0.0;
  s += (1.0 - mdx) * (1.0 - mdy) * __ldg(f + r0 + i);
  s += (1.0 - mdx) * mdy * __ldg(f + r1 + i);
  s += mdx * (1.0 - mdy) * __ldg(f + r0 + i1);
  s += mdx * mdy * __ldg(f + r1 + i1);
  return s;
}

// Per-marker projection geometry of one binning: the fractional offsets of the marker in its
// basic cell and in its cell-centre cell (the divisions of markerProjection.c:127-154, correctly
// rounded), the quadrant / nearest-node bits, and (product build) the two cells' corner weights.
struct GeoOut {
  double *gx0, *gy0, *gx1, *gy1;
  int *flags;  // bit0 qx, bit1 qy, bit2 mdx0>=.5, bit3 mdy0>=.5, bit4 mdx1>=.5, bit5 mdy1>=.5
  double *w0, *w1;
};

__device__ __forceinline__ void geometry_marker(const Params &P, double x, double y, int cx, int cy, const GeoOut &o,
                                                int64_t m) {
  if (cx < 0) {
    o.flags[m] = 0;
    return;
  }
  // basic cell (markerProjection.c:131-146, stagger 0)
  const double mdx0 = div_sp(x - P.x[cx], P.hx[cx], P.ix[cx]);
  const double mdy0 = div_sp(y - P.y[cy], P.hy[cy], P.iy[cy]);
  // cell-centre cell (findCellStag2D stagger -1, markerProjection.c:260-267, 128-143)
  const int qx = nonneg_bits(x) >= nonneg_bits(P.xc[cx + 1]);
  const int qy = nonneg_bits(y) >= nonneg_bits(P.yc[cy + 1]);
  const int sx = cx + qx, sy = cy + qy;
  const double mdx1 = div_sp(x - P.xc[sx], P.hxc[sx], P.ixc[sx]);
  const double mdy1 = div_sp(y - P.yc[sy], P.hyc[sy], P.iyc[sy]);
  const long long half = 0x3FE0000000000000LL;  // bits of 0.5; all offsets here are >= 0
  int f = qx | (qy << 1);
  f |= (nonneg_bits(mdx0) >= half) << 2;
  f |= (nonneg_bits(mdy0) >= half) << 3;
  f |= (nonneg_bits(mdx1) >= half) << 4;
  f |= (nonneg_bits(mdy1) >= half) << 5;
  o.gx0[m] = mdx0;
  o.gy0[m] = mdy0;
  o.gx1[m] = mdx1;
  o.gy1[m] = mdy1;
  o.flags[m] = f;
  if (o.w0) {  // the weights every later interpolation and projection of the step uses
    store_w4(o.w0, m, make_w4(mdx0, mdy0));
    store_w4(o.w1, m, make_w4(mdx1, mdy1));
  }
}

inline GeoOut geo_out(mic_ctx *ctx) {
  return GeoOut{ctx->geo[0], ctx->geo[1], ctx->geo[2], ctx->geo[3], ctx->geo_flags, ctx->wgt[0], ctx->wgt[1]};
}

}  // namespace mic
