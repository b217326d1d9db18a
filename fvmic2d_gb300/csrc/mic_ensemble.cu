// mic_ensemble.cu -- many independent marker-in-cell problems stepped together on one GPU.
//
// Members are ordinary contexts, each with its own stream.  One ensemble step forks from the
// ensemble stream to every member stream (events), issues each member's whole step (the same
// launches as mic_step without a residual read, so nothing waits on the host) and joins back.
// Small members then overlap on the GPU instead of running one after another.
//
// With graphs on, the fork / members / join sequence is captured once into CUDA graphs and each
// later step is a single graph launch.  A step's launches read the marker columns from one
// buffer of each double-buffered pair and leave them in the other (the binning's reorder), so
// the sequence alternates between two layouts: two graphs are captured, one per layout, and
// replays alternate between them while the host keeps each member's column pointers in step.
// A graph is re-captured when a member's settings change (materials, options, boundary values,
// creep configuration, launch shapes, marker count: the member's generation counter), when the
// time steps do, or when a member's column buffers are not where the graph expects them (the
// member was stepped, tuned or restored outside the ensemble since the last replay).
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "mic_internal.cuh"

struct mic_ensemble {
  int device;
  int n;
  std::vector<mic_ctx *> m;
  cudaStream_t stream;
  cudaEvent_t fork;
  std::vector<cudaEvent_t> join;
  // captured steps
  int have_graph;
  cudaGraphExec_t exec[2];
  int parity;
  std::vector<double> key_dt;  // dt_disp and dt_thermal per member at capture
  std::vector<long long> key_gen;
  std::vector<const void *> key_cols;  // per member and graph: the f64 column buffer it reads first
  int key_sub;
  long long graph_kernels[2];  // kernel launches inside each graph
  long long launches;          // kernel launches issued through this ensemble
  std::vector<int> order;      // members in the order their steps are issued (and captured)
};

namespace {

int fail(cudaError_t e) {
  mic_fail_cuda(nullptr, e);
  return MIC_ERR_CUDA;
}

// fork, every member's step, join: all asynchronous on the ensemble stream's timeline
int issue(mic_ensemble *E, const double *dt_disp, const double *dt_thermal, int sub) {
  cudaError_t ce = cudaEventRecord(E->fork, E->stream);
  if (ce != cudaSuccess) return fail(ce);
  for (int k = 0; k < E->n; ++k) {
    const int i = E->order[k];
    mic_ctx *c = E->m[i];
    if ((ce = cudaStreamWaitEvent(c->stream, E->fork, 0)) != cudaSuccess) return fail(ce);
    const long long l0 = c->launches;
    const int e = mic_step(c, dt_disp[i], dt_thermal[i], sub, nullptr);
    if (e) return e;
    E->launches += c->launches - l0;
    if ((ce = cudaEventRecord(E->join[i], c->stream)) != cudaSuccess) return fail(ce);
    if ((ce = cudaStreamWaitEvent(E->stream, E->join[i], 0)) != cudaSuccess) return fail(ce);
  }
  return MIC_OK;
}

void drop_graphs(mic_ensemble *E) {
  for (int q = 0; q < 2; ++q)
    if (E->have_graph) cudaGraphExecDestroy(E->exec[q]);
  E->have_graph = 0;
}

bool graph_current(const mic_ensemble *E, const double *dt_disp, const double *dt_thermal, int sub) {
  if (!E->have_graph || E->key_sub != sub) return false;
  for (int i = 0; i < E->n; ++i) {
    if (E->key_dt[2 * i] != dt_disp[i] || E->key_dt[2 * i + 1] != dt_thermal[i]) return false;
    if (E->key_gen[i] != E->m[i]->gen) return false;
    if (E->key_cols[2 * i + E->parity] != (const void *)E->m[i]->f64[0]) return false;
  }
  return true;
}

// the host side of a replayed step: the binning swapped each member's column buffers
void replayed(mic_ensemble *E) {
  for (int i = 0; i < E->n; ++i) {
    mic_ctx *c = E->m[i];
    if (c->n == 0) continue;
    const int nf = c->has_grain ? mic::C_F64_COUNT : mic::C_AOS_F64;
    for (int k = 0; k < nf; ++k) {
      double *t = c->f64[k];
      c->f64[k] = c->f64_alt[k];
      c->f64_alt[k] = t;
    }
    for (int k = 0; k < mic::C_I32_COUNT; ++k) {
      int *t = c->i32[k];
      c->i32[k] = c->i32_alt[k];
      c->i32_alt[k] = t;
    }
    mic_invalidate_sort(c);
  }
}

int capture(mic_ensemble *E, const double *dt_disp, const double *dt_thermal, int sub) {
  drop_graphs(E);
  E->key_cols.assign(2 * E->n, nullptr);
  for (int q = 0; q < 2; ++q) {
    for (int i = 0; i < E->n; ++i) E->key_cols[2 * i + q] = E->m[i]->f64[0];
    std::vector<int> prof(E->n);
    for (int i = 0; i < E->n; ++i) {  // no per-launch timing events inside a graph
      prof[i] = E->m[i]->prof_on;
      E->m[i]->prof_on = 0;
    }
    cudaError_t ce = cudaStreamBeginCapture(E->stream, cudaStreamCaptureModeRelaxed);
    if (ce != cudaSuccess) return fail(ce);
    const long long l0 = E->launches;
    int e = issue(E, dt_disp, dt_thermal, sub);
    cudaGraph_t g = nullptr;
    ce = cudaStreamEndCapture(E->stream, &g);
    for (int i = 0; i < E->n; ++i) E->m[i]->prof_on = prof[i];
    E->graph_kernels[q] = E->launches - l0;
    E->launches = l0;
    if (e) {
      if (g) cudaGraphDestroy(g);
      if (q == 1) cudaGraphExecDestroy(E->exec[0]);
      return e;
    }
    if (ce != cudaSuccess) return fail(ce);
    ce = cudaGraphInstantiate(&E->exec[q], g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      if (q == 1) cudaGraphExecDestroy(E->exec[0]);
      return fail(ce);
    }
  }
  // two captured steps swapped every member's buffers twice: the host view is unchanged
  E->have_graph = 1;
  E->parity = 0;
  E->key_sub = sub;
  E->key_dt.assign(2 * E->n, 0.0);
  E->key_gen.assign(E->n, 0);
  for (int i = 0; i < E->n; ++i) {
    E->key_dt[2 * i] = dt_disp[i];
    E->key_dt[2 * i + 1] = dt_thermal[i];
    E->key_gen[i] = E->m[i]->gen;
  }
  return MIC_OK;
}

}  // namespace

extern "C" int mic_ensemble_create(mic_ensemble **out, mic_ctx *const *members, int n_members) {
  if (!out || !members || n_members < 1) return MIC_ERR_ARG;
  for (int i = 0; i < n_members; ++i)
    if (!members[i] || members[i]->device != members[0]->device) return MIC_ERR_ARG;
  for (int i = 0; i < n_members; ++i)
    for (int j = 0; j < i; ++j)
      if (members[i] == members[j] || members[i]->stream == members[j]->stream) return MIC_ERR_ARG;
  mic_ensemble *E = new (std::nothrow) mic_ensemble();
  if (!E) return MIC_ERR_NOMEM;
  E->device = members[0]->device;
  E->n = n_members;
  E->m.assign(members, members + n_members);
  E->join.assign(n_members, nullptr);
  E->order.resize(n_members);
  for (int i = 0; i < n_members; ++i) E->order[i] = i;
  cudaSetDevice(E->device);
  bool ok = cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&E->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < n_members; ++i)
    ok = cudaEventCreateWithFlags(&E->join[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    delete E;
    return MIC_ERR_CUDA;
  }
  *out = E;
  return MIC_OK;
}

extern "C" int mic_ensemble_destroy(mic_ensemble *E) {
  if (!E) return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  cudaStreamSynchronize(E->stream);
  drop_graphs(E);
  for (auto ev : E->join)
    if (ev) cudaEventDestroy(ev);
  cudaEventDestroy(E->fork);
  cudaStreamDestroy(E->stream);
  delete E;
  return MIC_OK;
}

// One step of every member (dt_disp[i], dt_thermal[i]; subgrid stress changes on or off).
// Asynchronous: returns once the work is queued; mic_ensemble_synchronize waits for it.  With
// use_graph, the first call (and any call after a member's settings or the time steps changed)
// runs the step directly and captures the graphs the following calls launch.
extern "C" int mic_ensemble_step(mic_ensemble *E, const double *dt_disp, const double *dt_thermal,
                                 int subgrid_stress, int use_graph) {
  if (!E || !dt_disp || !dt_thermal) return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  if (!use_graph) {
    drop_graphs(E);
    return issue(E, dt_disp, dt_thermal, subgrid_stress);
  }
  if (graph_current(E, dt_disp, dt_thermal, subgrid_stress)) {
    // the graph runs after whatever the caller queued on member streams (nodal uploads), and
    // member streams see its results
    cudaError_t ce;
    for (int i = 0; i < E->n; ++i) {
      if ((ce = cudaEventRecord(E->join[i], E->m[i]->stream)) != cudaSuccess) return fail(ce);
      if ((ce = cudaStreamWaitEvent(E->stream, E->join[i], 0)) != cudaSuccess) return fail(ce);
    }
    if ((ce = cudaGraphLaunch(E->exec[E->parity], E->stream)) != cudaSuccess) return fail(ce);
    if ((ce = cudaEventRecord(E->fork, E->stream)) != cudaSuccess) return fail(ce);
    for (int i = 0; i < E->n; ++i)
      if ((ce = cudaStreamWaitEvent(E->m[i]->stream, E->fork, 0)) != cudaSuccess) return fail(ce);
    E->launches += E->graph_kernels[E->parity];
    replayed(E);
    E->parity ^= 1;
    return MIC_OK;
  }
  int e = issue(E, dt_disp, dt_thermal, subgrid_stress);  // this call's step, run directly
  if (e) return e;
  cudaError_t ce = cudaStreamSynchronize(E->stream);  // scratch sized, nothing in flight
  if (ce != cudaSuccess) return fail(ce);
  return capture(E, dt_disp, dt_thermal, subgrid_stress);
}

extern "C" int mic_ensemble_synchronize(mic_ensemble *E) {
  if (!E) return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  cudaError_t ce = cudaStreamSynchronize(E->stream);
  return ce == cudaSuccess ? MIC_OK : fail(ce);
}

extern "C" int mic_ensemble_launch_count(mic_ensemble *E, int64_t *launches, int64_t *graph_kernels) {
  if (!E) return MIC_ERR_ARG;
  if (launches) *launches = E->launches;
  if (graph_kernels) *graph_kernels = E->have_graph ? E->graph_kernels[0] : 0;
  return MIC_OK;
}

extern "C" int mic_ensemble_get_stream(mic_ensemble *E, void **stream) {
  if (!E || !stream) return MIC_ERR_ARG;
  *stream = (void *)E->stream;
  return MIC_OK;
}

// Launch shapes and the member schedule, measured on the ensemble's own members: each member's
// kernels get their block sizes from mic_autotune (member by member), then the order in which
// the members' steps are issued into the step (and its captured graphs) is chosen among: as
// given, largest member first, smallest first, by timing `steps` pairs of graph replays of each
// from the same saved state.  Every member's state is put back at the end.  order_out (n ints,
// may be NULL) receives the chosen order.
extern "C" int mic_ensemble_autotune(mic_ensemble *E, const double *dt_disp, const double *dt_thermal,
                                     int subgrid_stress, int steps, int *order_out) {
  if (!E || !dt_disp || !dt_thermal || steps < 0) return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  if (steps == 0) steps = 1;
  int e = MIC_OK;
  for (int i = 0; i < E->n && !e; ++i) e = mic_autotune(E->m[i], dt_disp[i], dt_thermal[i], subgrid_stress, 1, nullptr);
  if (e) return e;
  std::vector<void *> saved(E->n, nullptr);
  for (int i = 0; i < E->n && !e; ++i) e = mic_state_save(E->m[i], &saved[i]);
  std::vector<std::vector<int>> cand(3, E->order);
  for (int i = 0; i < E->n; ++i) cand[0][i] = i;
  cand[1] = cand[0];
  std::stable_sort(cand[1].begin(), cand[1].end(), [&](int a, int b) { return E->m[a]->n > E->m[b]->n; });
  cand[2] = cand[0];
  std::stable_sort(cand[2].begin(), cand[2].end(), [&](int a, int b) { return E->m[a]->n < E->m[b]->n; });
  const std::vector<int> before = E->order;
  int best = -1;
  float best_ms = 0.f;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (!e && (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess)) e = MIC_ERR_CUDA;
  for (int c = 0; c < (int)cand.size() && !e; ++c) {
    E->order = cand[c];
    drop_graphs(E);
    for (int i = 0; i < E->n && !e; ++i) e = mic_state_restore(E->m[i], saved[i]);
    if (e) break;
    for (int w = 0; w < 3 && !e; ++w) e = mic_ensemble_step(E, dt_disp, dt_thermal, subgrid_stress, 1);  // capture
    if (e) break;
    if (cudaEventRecord(t0, E->stream) != cudaSuccess) e = MIC_ERR_CUDA;
    for (int s = 0; s < 2 * steps && !e; ++s) e = mic_ensemble_step(E, dt_disp, dt_thermal, subgrid_stress, 1);
    if (e) break;
    float ms = 0.f;
    if (cudaEventRecord(t1, E->stream) != cudaSuccess || cudaEventSynchronize(t1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, t0, t1) != cudaSuccess) {
      e = MIC_ERR_CUDA;
      break;
    }
    if (best < 0 || ms < best_ms) {
      best = c;
      best_ms = ms;
    }
  }
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  drop_graphs(E);
  E->order = (!e && best >= 0) ? cand[best] : before;
  int e2 = MIC_OK;
  for (int i = 0; i < E->n; ++i) {
    if (saved[i] && !e2) e2 = mic_state_restore(E->m[i], saved[i]);
    if (cudaStreamSynchronize(E->m[i]->stream) != cudaSuccess && !e2) e2 = MIC_ERR_CUDA;
    mic_state_free(saved[i]);
  }
  if (e || e2) return e ? e : e2;
  if (order_out)
    for (int k = 0; k < E->n; ++k) order_out[k] = E->order[k];
  return MIC_OK;
}
