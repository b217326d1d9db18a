// mic_ensemble.cu -- many independent marker-in-cell problems stepped together on one GPU.
//
// Members are ordinary contexts, each with its own stream.  One ensemble step forks from the
// ensemble stream to every member stream (events), issues each member's whole step (the same
// launches as mic_step without a residual read, so nothing waits on the host) and joins back.
// Small members then overlap on the GPU instead of running one after another.
//
// Batched (the default): a step's marker passes run as one kernel per pass over many members
// instead of one per member.  A step is cut into segments at its marker passes
// (mic_step_segment); each segment's own launches (binning, projections, node kernels) are
// issued on every member's stream, the members join their batch group's stream, one batched
// kernel per pass walks the group's work table of (member, tile) pairs, and the members fork
// again.  With several groups (members dealt by marker count), one group's batched passes
// overlap the other groups' member work, since a pass waits for its slowest member.  The table (the
// members' launch arguments and their tile offsets) is written on the host and copied into a
// device buffer: once per captured graph (the graph reads it at every replay), or by an
// asynchronous copy before each pass of a step run directly (two alternating buffers).  The
// tile size, the persistent / one-tile-per-block grid and the block-to-tile schedule come from
// mic_ensemble_set_schedule or mic_ensemble_autotune.  Per-member (no groups): each member's
// whole step on its own stream, between one fork and one join.
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

constexpr int kMaxGroups = 8;

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
  // batched marker passes: `groups` batch groups (0: per-member steps), each with its own stream,
  // fork event, completion event and batch; members are dealt to the groups by marker count
  int groups;
  mic::BatchShape shape[mic::BP_COUNT];
  cudaStream_t gstream[kMaxGroups];
  cudaEvent_t gfork[kMaxGroups], gdone[kMaxGroups];
  mic_batch *gbatch[kMaxGroups];
  size_t table_cap;
  // work tables: slot 0, 1 the captured graphs of either parity; 2, 3 steps run directly (in turn)
  unsigned char *h_table[4], *d_table[4];
  size_t table_used[4];
  cudaEvent_t table_ev[2];  // end of the last direct step that used slot 2 + k
  int table_ev_live[2];
  int direct_next;
};

constexpr int kSlotDirect = 2;
// default walk of a batched pass: tiles of 4 blocks' worth of markers, persistent grid, blocks
// taking the next tile from a shared counter
constexpr mic::BatchShape kDefaultShape = {4, 1, 2};
// default batch groups: a pass waits for its group's slowest member, and the tensor-core yield
// pass fills every SM's registers, so a single group leaves the other streams' memory-bound work
// no room beside it; four groups interleave their phases
constexpr int kDefaultGroups = 4;

namespace {

int fail(cudaError_t e) {
  mic_fail_cuda(nullptr, e);
  return MIC_ERR_CUDA;
}

int ensure_tables(mic_ensemble *E) {
  if (E->h_table[0]) return MIC_OK;
  // every group's table in its own region: at most the whole ensemble's bound plus one empty
  // table's overhead per further group
  E->table_cap = mic_batch_table_bound(E->n) + kMaxGroups * mic_batch_table_bound(0);
  for (int k = 0; k < 4; ++k) {
    cudaError_t ce = cudaHostAlloc((void **)&E->h_table[k], E->table_cap, cudaHostAllocDefault);
    if (ce == cudaSuccess) ce = cudaMalloc((void **)&E->d_table[k], E->table_cap);
    if (ce != cudaSuccess) return fail(ce);
  }
  return MIC_OK;
}

// members dealt to the batch groups: largest marker count first, each to the group with the
// fewest markers so far (ties: the lower group); each group keeps the issue order
std::vector<std::vector<int>> group_members(const mic_ensemble *E) {
  const int G = E->groups < 1 ? 1 : (E->groups > E->n ? E->n : E->groups);
  std::vector<int> by_size = E->order;
  std::stable_sort(by_size.begin(), by_size.end(), [&](int a, int b) { return E->m[a]->n > E->m[b]->n; });
  std::vector<int64_t> load(G, 0);
  std::vector<int> group_of(E->n, 0);
  for (int i : by_size) {
    int g = 0;
    for (int h = 1; h < G; ++h)
      if (load[h] < load[g]) g = h;
    group_of[i] = g;
    load[g] += E->m[i]->n;
  }
  std::vector<std::vector<int>> out(G);
  for (int i : E->order) out[group_of[i]].push_back(i);
  return out;
}

cudaError_t join_group(mic_ensemble *E, const std::vector<int> &mem, cudaStream_t s) {
  cudaError_t ce = cudaSuccess;
  for (size_t k = 0; k < mem.size() && ce == cudaSuccess; ++k) {
    ce = cudaEventRecord(E->join[mem[k]], E->m[mem[k]]->stream);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(s, E->join[mem[k]], 0);
  }
  return ce;
}

cudaError_t fork_group(mic_ensemble *E, const std::vector<int> &mem, cudaStream_t s, cudaEvent_t ev) {
  cudaError_t ce = cudaEventRecord(ev, s);
  for (size_t k = 0; k < mem.size() && ce == cudaSuccess; ++k) ce = cudaStreamWaitEvent(E->m[mem[k]]->stream, ev, 0);
  return ce;
}

// One step with batched marker passes; its work tables go to `slot` (a graph being captured, or
// kSlotDirect: the next direct buffer, copied inside the step), one region per group.  Every
// group runs its own chain -- its members' segments on their streams, a join into the group
// stream, the batched passes, a fork back -- beside the other groups; the ensemble stream forks
// the groups at the start and joins them at the end.
int issue_batched(mic_ensemble *E, const double *dt_disp, const double *dt_thermal, int sub, int slot) {
  int e = ensure_tables(E);
  if (e) return e;
  cudaError_t ce;
  int ev = -1;
  if (slot == kSlotDirect) {
    ev = E->direct_next;
    E->direct_next ^= 1;
    slot = kSlotDirect + ev;
    // the host buffer is rewritten below: the step that last copied out of it must be done
    if (E->table_ev_live[ev] && (ce = cudaEventSynchronize(E->table_ev[ev])) != cudaSuccess) return fail(ce);
  }
  const bool copy = ev >= 0;
  const std::vector<std::vector<int>> gm = group_members(E);
  const int G = (int)gm.size();
  std::vector<size_t> off(G), end(G);
  size_t base = 0;
  for (int g = 0; g < G; ++g) {
    off[g] = base;
    base += mic_batch_table_bound((int)gm[g].size());
    end[g] = base;
  }
  if ((ce = cudaEventRecord(E->fork, E->stream)) != cudaSuccess) return fail(ce);
  for (int g = 0; g < G && !e; ++g) {
    if ((ce = cudaStreamWaitEvent(E->gstream[g], E->fork, 0)) != cudaSuccess ||
        (ce = fork_group(E, gm[g], E->gstream[g], E->gfork[g])) != cudaSuccess)
      e = fail(ce);
  }
  for (int seg = 0; seg < mic::kStepSegments && !e; ++seg) {
    for (int g = 0; g < G && !e; ++g) {
      for (size_t k = 0; k < gm[g].size() && !e; ++k) {
        const int i = gm[g][k];
        mic_ctx *c = E->m[i];
#ifdef MIC_EXACT
        const int wz_known = 0;
#else
        const int wz_known = c->n > 0;  // as mic_step
#endif
        const long long l0 = c->launches;
        e = mic_step_segment(c, seg, dt_disp[i], dt_thermal[i], sub, wz_known, E->gbatch[g]);
        E->launches += c->launches - l0;
      }
      if (e || mic_batch_empty(E->gbatch[g])) continue;
      if ((ce = join_group(E, gm[g], E->gstream[g])) != cudaSuccess) {
        e = fail(ce);
        break;
      }
      // the group's region is sized for its members: the table cannot run into the next group's
      e = mic_batch_launch(E->gbatch[g], E->shape, E->h_table[slot], E->d_table[slot], &off[g], end[g],
                           copy ? 1 : 0, E->gstream[g], &E->launches);
      if (!e && (ce = fork_group(E, gm[g], E->gstream[g], E->gfork[g])) != cudaSuccess) e = fail(ce);
    }
  }
  for (int g = 0; g < G; ++g) {
    mic_batch_clear(E->gbatch[g]);
    if ((ce = join_group(E, gm[g], E->gstream[g])) != cudaSuccess && !e) e = fail(ce);
    if ((ce = cudaEventRecord(E->gdone[g], E->gstream[g])) != cudaSuccess && !e) e = fail(ce);
    if ((ce = cudaStreamWaitEvent(E->stream, E->gdone[g], 0)) != cudaSuccess && !e) e = fail(ce);
  }
  E->table_used[slot] = base;
  if (copy && !e) {
    if ((ce = cudaEventRecord(E->table_ev[ev], E->stream)) != cudaSuccess) return fail(ce);
    E->table_ev_live[ev] = 1;
  }
  return e;
}

// fork, every member's step, join: all asynchronous on the ensemble stream's timeline
int issue(mic_ensemble *E, const double *dt_disp, const double *dt_thermal, int sub, int slot = kSlotDirect) {
  if (E->groups > 0) return issue_batched(E, dt_disp, dt_thermal, sub, slot);
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
    int e = issue(E, dt_disp, dt_thermal, sub, q);
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
    // the graph's batched kernels read the work table written while it was captured: copy it
    // into the graph's own device buffer now (nothing in flight reads that buffer)
    if (E->groups > 0 && E->table_used[q] > 0 &&
        (ce = cudaMemcpy(E->d_table[q], E->h_table[q], E->table_used[q], cudaMemcpyHostToDevice)) != cudaSuccess) {
      cudaGraphExecDestroy(E->exec[q]);
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
  E->groups = kDefaultGroups;
  for (int p = 0; p < mic::BP_COUNT; ++p) E->shape[p] = kDefaultShape;
  cudaSetDevice(E->device);
  bool ok = cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&E->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&E->table_ev[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&E->table_ev[1], cudaEventDisableTiming) == cudaSuccess;
  for (int g = 0; ok && g < kMaxGroups; ++g)
    ok = (E->gbatch[g] = mic_batch_new()) != nullptr &&
         cudaStreamCreateWithFlags(&E->gstream[g], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&E->gfork[g], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&E->gdone[g], cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < n_members; ++i)
    ok = cudaEventCreateWithFlags(&E->join[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    mic_ensemble_destroy(E);
    return MIC_ERR_CUDA;
  }
  *out = E;
  return MIC_OK;
}

extern "C" int mic_ensemble_destroy(mic_ensemble *E) {
  if (!E) return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  if (E->stream) cudaStreamSynchronize(E->stream);
  drop_graphs(E);
  for (auto ev : E->join)
    if (ev) cudaEventDestroy(ev);
  if (E->fork) cudaEventDestroy(E->fork);
  for (int k = 0; k < 2; ++k)
    if (E->table_ev[k]) cudaEventDestroy(E->table_ev[k]);
  for (int k = 0; k < 4; ++k) {
    if (E->h_table[k]) cudaFreeHost(E->h_table[k]);
    if (E->d_table[k]) cudaFree(E->d_table[k]);
  }
  for (int g = 0; g < kMaxGroups; ++g) {
    if (E->gstream[g]) cudaStreamDestroy(E->gstream[g]);
    if (E->gfork[g]) cudaEventDestroy(E->gfork[g]);
    if (E->gdone[g]) cudaEventDestroy(E->gdone[g]);
    mic_batch_free(E->gbatch[g]);
  }
  if (E->stream) cudaStreamDestroy(E->stream);
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

// How a step runs its marker passes: `groups` batch groups (0: each member's own kernels on its
// stream; 1..kMaxGroups: members dealt to that many groups by marker count, one kernel per pass
// per group), and for the batched kernels the tile size in blocks' worth of markers, persistent
// grid or one block per tile, and on a persistent grid the walk: tiles round-robin (chunked 0),
// one contiguous run per block (1) or the next tile from a shared counter (2).  The surrogate
// passes always take one-block tiles from a counter on a persistent grid (a block stages the
// network again only when a tile reads another copy).
extern "C" int mic_ensemble_set_schedule(mic_ensemble *E, int groups, int tile_mult, int persistent, int chunked) {
  if (!E || groups < 0 || groups > kMaxGroups || tile_mult < 1 || tile_mult > 64 || chunked < 0 || chunked > 2)
    return MIC_ERR_ARG;
  cudaSetDevice(E->device);
  drop_graphs(E);
  E->groups = groups;
  for (int p = 0; p < mic::BP_COUNT; ++p) E->shape[p] = {tile_mult, persistent ? 1 : 0, chunked};
  return MIC_OK;
}

extern "C" int mic_ensemble_get_schedule(mic_ensemble *E, int *groups, int *tile_mult, int *persistent,
                                         int *chunked) {
  if (!E) return MIC_ERR_ARG;
  if (groups) *groups = E->groups;
  if (tile_mult) *tile_mult = E->shape[0].mult;
  if (persistent) *persistent = E->shape[0].persistent;
  if (chunked) *chunked = E->shape[0].chunked;
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
  std::vector<int> given(E->n), big(E->n), small(E->n);
  for (int i = 0; i < E->n; ++i) given[i] = i;
  big = given;
  std::stable_sort(big.begin(), big.end(), [&](int a, int b) { return E->m[a]->n > E->m[b]->n; });
  small = given;
  std::stable_sort(small.begin(), small.end(), [&](int a, int b) { return E->m[a]->n < E->m[b]->n; });
  struct Cand {
    std::vector<int> order;
    int groups;
    mic::BatchShape shape;
  };
  // per-member steps in three issue orders, then batched passes in 1, 2, 4 and 8 groups, each
  // with three walks (one block per tile; persistent grids over tiles of four blocks' worth taken
  // as contiguous runs or from a shared counter)
  std::vector<Cand> cand;
  for (const auto *o : {&given, &big, &small}) cand.push_back({*o, 0, kDefaultShape});
  const mic::BatchShape walks[3] = {{1, 0, 0}, {4, 1, 1}, {4, 1, 2}};
  for (int g = 1; g <= kMaxGroups; g *= 2)
    if (g == 1 || g <= E->n)
      for (const auto &w : walks) cand.push_back({given, g, w});
  const std::vector<int> before = E->order;
  const int groups_before = E->groups;
  mic::BatchShape shape_before[mic::BP_COUNT];
  for (int p = 0; p < mic::BP_COUNT; ++p) shape_before[p] = E->shape[p];
  int best = -1;
  float best_ms = 0.f;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (!e && (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess)) e = MIC_ERR_CUDA;
  for (int c = 0; c < (int)cand.size() && !e; ++c) {
    E->order = cand[c].order;
    E->groups = cand[c].groups;
    for (int p = 0; p < mic::BP_COUNT; ++p) E->shape[p] = cand[c].shape;
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
  if (!e && best >= 0) {
    E->order = cand[best].order;
    E->groups = cand[best].groups;
    for (int p = 0; p < mic::BP_COUNT; ++p) E->shape[p] = cand[best].shape;
  } else {
    E->order = before;
    E->groups = groups_before;
    for (int p = 0; p < mic::BP_COUNT; ++p) E->shape[p] = shape_before[p];
  }
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
