// mic_autotune.cu -- launch shapes picked on the context's own workload.
//
// The marker-parallel kernels of a step (TuneId) are launched with one block size each.  Which
// size runs fastest depends on the kernel's registers and on the workload (marker count, how the
// markers sit in their cells, the materials), so mic_autotune measures it: it saves the marker
// columns and nodal fields, and for every candidate size restores them, runs one untimed step and
// then `steps` timed steps with an event pair around every launch, and keeps, kernel by kernel,
// the size with the least time.  The saved state is put back at the end, so tuning leaves the
// simulation where it was; the choices stay in the context (mic_get_tuning / mic_set_tuning
// carry them to another context of the same workload).
#include <cstring>
#include <new>
#include <vector>

#include "mic_internal.cuh"

using namespace mic;

namespace {

// profiling names of the tuned kernels, in TuneId order
const char *const kTuneName[TU_COUNT] = {"k_advect",          "k_strain_pressure",      "k_yield",
                                         "k_subgrid_stress_markers", "k_update_marker_stress",
                                         "k_subgridT_markers", "k_subgridT_apply",       "k_reorder",
                                         "k_find_cells",      "k_update_rho"};
constexpr int kCandidates[] = {128, 256, 512};

struct Snapshot {
  std::vector<void *> bufs;
  int64_t n = 0;
};

void snapshot_free(Snapshot &s) {
  for (void *p : s.bufs) cudaFree(p);
  s.bufs.clear();
}

// copies of the marker columns [0, n) and of the nodal fields
int snapshot_take(mic_ctx *ctx, Snapshot &s) {
  s.n = ctx->n;
  const size_t nn = (size_t)ctx->P.NX * ctx->P.NY;
  for (int c = 0; c < C_F64_COUNT + C_I32_COUNT + MIC_NF_COUNT; ++c) {
    const bool f = c < C_F64_COUNT, i = !f && c < C_F64_COUNT + C_I32_COUNT;
    const size_t bytes = f ? sizeof(double) * (size_t)s.n : i ? sizeof(int) * (size_t)s.n : sizeof(double) * nn;
    void *p = nullptr;
    if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) {
      snapshot_free(s);
      return MIC_ERR_NOMEM;
    }
    s.bufs.push_back(p);
    const void *src = f ? (const void *)ctx->f64[c]
                        : i ? (const void *)ctx->i32[c - C_F64_COUNT] : (const void *)ctx->nodal[c - C_F64_COUNT - C_I32_COUNT];
    if (bytes) MIC_CUDA_TRY(cudaMemcpyAsync(p, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  return MIC_OK;
}

int snapshot_restore(mic_ctx *ctx, const Snapshot &s) {
  if (ctx->n != s.n) ctx->gen++;  // launch grids follow the marker count
  ctx->n = s.n;
  const size_t nn = (size_t)ctx->P.NX * ctx->P.NY;
  for (int c = 0; c < (int)s.bufs.size(); ++c) {
    const bool f = c < C_F64_COUNT, i = !f && c < C_F64_COUNT + C_I32_COUNT;
    const size_t bytes = f ? sizeof(double) * (size_t)s.n : i ? sizeof(int) * (size_t)s.n : sizeof(double) * nn;
    void *dst = f ? (void *)ctx->f64[c] : i ? (void *)ctx->i32[c - C_F64_COUNT] : (void *)ctx->nodal[c - C_F64_COUNT - C_I32_COUNT];
    if (bytes) MIC_CUDA_TRY(cudaMemcpyAsync(dst, s.bufs[c], bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  mic_invalidate_sort(ctx);
  return MIC_OK;
}

// per-kernel totals of the recorded launches, by TuneId (negative where a kernel did not run)
int tuned_times(mic_ctx *ctx, double *t) {
  char names[128 * 48];
  double tot[128];
  int nk = 0;
  int e = mic_profile_read(ctx, 128, names, tot, nullptr, &nk);
  if (e) return e;
  for (int id = 0; id < TU_COUNT; ++id) {
    t[id] = -1.0;
    for (int k = 0; k < nk && k < 128; ++k)
      if (strcmp(names + 48 * k, kTuneName[id]) == 0) t[id] = tot[k];
  }
  return MIC_OK;
}

}  // namespace

// saved marker columns and nodal fields of a context (ensemble tuning)
int mic_state_save(mic_ctx *ctx, void **handle) {
  Snapshot *s = new (std::nothrow) Snapshot;
  if (!s) return MIC_ERR_NOMEM;
  const int e = snapshot_take(ctx, *s);
  if (e) {
    delete s;
    return e;
  }
  *handle = s;
  return MIC_OK;
}
int mic_state_restore(mic_ctx *ctx, void *handle) { return snapshot_restore(ctx, *(Snapshot *)handle); }
void mic_state_free(void *handle) {
  if (!handle) return;
  snapshot_free(*(Snapshot *)handle);
  delete (Snapshot *)handle;
}

extern "C" int mic_autotune(mic_ctx *ctx, double dt_disp, double dt_thermal, int subgrid_stress, int steps,
                            int *chosen) {
  if (!ctx || steps < 0) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (steps == 0) steps = 1;
  const int prof_was = ctx->prof_on ? ctx->prof_cap : 0;
  int saved[TU_COUNT];
  memcpy(saved, ctx->tune_bs, sizeof(saved));
  double best_t[TU_COUNT];
  int best_b[TU_COUNT];
  for (int id = 0; id < TU_COUNT; ++id) {
    best_t[id] = -1.0;
    best_b[id] = saved[id];
  }
  Snapshot snap;
  int e = snapshot_take(ctx, snap);
  for (int b : kCandidates) {
    if (e) break;
    for (int id = 0; id < TU_COUNT; ++id) ctx->tune_bs[id] = b;
    if ((e = snapshot_restore(ctx, snap))) break;
    if ((e = mic_profile_enable(ctx, 0))) break;
    if ((e = mic_step(ctx, dt_disp, dt_thermal, subgrid_stress, nullptr))) break;
    if ((e = mic_profile_enable(ctx, 64 * steps))) break;
    for (int s = 0; s < steps && !e; ++s) e = mic_step(ctx, dt_disp, dt_thermal, subgrid_stress, nullptr);
    if (e) break;
    double t[TU_COUNT];
    if ((e = tuned_times(ctx, t))) break;
    for (int id = 0; id < TU_COUNT; ++id)
      if (t[id] >= 0.0 && (best_t[id] < 0.0 || t[id] < best_t[id])) {
        best_t[id] = t[id];
        best_b[id] = b;
      }
  }
  // the caller's state and profiling back, whatever happened above
  int e2 = snap.bufs.empty() ? MIC_OK : snapshot_restore(ctx, snap);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess && !e2) e2 = MIC_ERR_CUDA;
  snapshot_free(snap);
  mic_profile_enable(ctx, prof_was);
  ctx->gen++;  // launch shapes (and, through the restores, buffers) changed: captured graphs are stale
  if (e || e2) {
    memcpy(ctx->tune_bs, saved, sizeof(saved));
    return e ? e : e2;
  }
  memcpy(ctx->tune_bs, best_b, sizeof(best_b));
  if (chosen)
    for (int id = 0; id < TU_COUNT; ++id) chosen[id] = tuned_block(ctx, id);
  return MIC_OK;
}

extern "C" int mic_get_tuning(mic_ctx *ctx, int *block, int count) {
  if (!ctx || !block || count < 0) return MIC_ERR_ARG;
  for (int id = 0; id < count && id < TU_COUNT; ++id) block[id] = tuned_block(ctx, id);
  return MIC_OK;
}

extern "C" int mic_set_tuning(mic_ctx *ctx, const int *block, int count) {
  if (!ctx || !block || count < 0) return MIC_ERR_ARG;
  for (int id = 0; id < count && id < TU_COUNT; ++id)
    if (block[id] != 0 && block[id] != 128 && block[id] != 256 && block[id] != 512) return MIC_ERR_ARG;
  for (int id = 0; id < count && id < TU_COUNT; ++id) ctx->tune_bs[id] = block[id];
  ctx->gen++;  // captured graphs hold the old launch shapes
  return MIC_OK;
}
