// mic_timestep.cu -- one time step of fvmic2d's subduction model (main_subduction.c:227-460)
// on the device, without PETSc: marker density control, the plasticity iterations around the
// Stokes solve, the sub-grid stress and stress updates, the thermal solve (repeated with a
// shorter step when the temperature changes too much) and the marker advection.  Every stage is
// the library's own entry point for the reference routine of the same name; the linear systems
// are assembled and solved on the device (mic_systems.cu, mic_band_lu.cu).  Nodal fields and
// markers stay on the device; only scalars (time steps, flags, maxima) come back to the host,
// where main_subduction's control flow runs.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "mic_internal.cuh"

using namespace mic;

namespace {

// VecNorm(thisT - lastT, NORM_INFINITY) (main:387-390), NaN entries skipped
__global__ void k_temp_change(const double *__restrict__ thisT, const double *__restrict__ lastT, int64_t nn,
                              double *part) {
  __shared__ double sm[256];
  double m = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
    const double d = fabs(thisT[k] - lastT[k]);
    if (d > m) m = d;
  }
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s && sm[threadIdx.x + s] > sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// adiabaticHeating (adiabaticHeating.c:24-43): each marker's alpha T VY rho gy, in the binned
// column order (out-of-domain markers are in no cell and contribute nothing)
__global__ void k_adiabatic_values(const int *__restrict__ cellX, const int *__restrict__ mat,
                                   const double *__restrict__ T, const double *__restrict__ VY, mic_materials M,
                                   double gy, int64_t n, double *v) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (m >= n) return;
  if (cellX[m] == -1) {
    v[m] = 0.0;
    return;
  }
  const int mt = mat[m];
  v[m] = M.materialAlpha[mt] * T[m] * VY[m] * M.materialRho[mt] * gy;
}

// VecAXPY(nodal_heating, 1.0, ha) (main_subduction.c:377)
__global__ void k_add_heating(double *heat, const double *__restrict__ ha, int64_t nn) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < nn) heat[k] = heat[k] + 1.0 * ha[k];
}

int max_temp_change(mic_ctx *ctx, double *out) {
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  constexpr int kParts = 64;
  double *part = ctx->red_buf;  // reduction scratch of the context (at least 64 entries)
  {
    MIC_KERNEL(ctx, "k_temp_change");
    k_temp_change<<<kParts, 256, 0, ctx->stream>>>(ctx->nodal[MIC_NF_THIST], ctx->nodal[MIC_NF_LASTT], nn, part);
  }
  double h[kParts];
  MIC_CUDA_TRY(cudaMemcpyAsync(h, part, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  double m = 0.0;
  for (double v : h)
    if (v > m) m = v;
  *out = m;
  return MIC_OK;
}

// main:381-384 / 396-399: heating into the right-hand side, boundary values of lastT, assembly,
// solve (the solution is thisT)
int thermal_solve(mic_ctx *ctx, const mic_timestep_options &o, double dt) {
  int e = mic_enforce_thermal_bcs(ctx, &o.sub);
  if (!e) e = mic_form_thermal_system(ctx, &o.sub, dt, 0);
  if (!e) e = mic_linear_solve(ctx, 1);
  return e;
}

}  // namespace

extern "C" int mic_adiabatic_heating(mic_ctx *ctx, double gy) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  int e = mic_ensure_sorted(ctx);
  if (e) return e;
  const int64_t nn = (int64_t)ctx->P.NX * ctx->P.NY;
  if (ctx->n > 0) {
    MIC_KERNEL(ctx, "k_adiabatic_values");
    k_adiabatic_values<<<grid_for(ctx->n), kBlock, 0, ctx->stream>>>(ctx->i32[C_CELLX], ctx->i32[C_MAT], ctx->f64[C_T],
                                                                     ctx->f64[C_VY], ctx->mat, gy, ctx->n, ctx->scr1);
  }
  // the markers' basic-node projection, weights (1 - mdx)(1 - mdy) etc., divided by their sum
  if ((e = mic_project_scalar(ctx, ctx->scr1, 0, ctx->node_scr[5]))) return e;
  {
    MIC_KERNEL(ctx, "k_add_heating");
    k_add_heating<<<grid_for(nn), kBlock, 0, ctx->stream>>>(ctx->nodal[MIC_NF_HEATING], ctx->node_scr[5], nn);
  }
  MIC_CUDA_TRY(cudaGetLastError());
  return MIC_OK;
}

#define MIC_TRY(x)           \
  do {                       \
    const int _e = (x);      \
    if (_e) return _e;       \
  } while (0)

extern "C" int mic_subduction_timestep(mic_ctx *ctx, const mic_timestep_options *o, double elapsed_time,
                                       mic_timestep_report *rep) {
  if (ctx && ctx->P.xper) return MIC_ERR_BC;  // grids periodic in x: the marker path only
  if (!ctx || !o || !rep) return MIC_ERR_ARG;
  if (ctx->red_cap < 64) return MIC_ERR_ARG;
  cudaSetDevice(ctx->device);
  *rep = mic_timestep_report{};
  int64_t n = 0;
  // main:241-250: cells, density control, cells
  MIC_TRY(mic_find_marker_cells(ctx, &n));
  if (o->densityControl) {
    MIC_TRY(mic_check_marker_density(ctx, &o->density, &rep->markers_added, &rep->markers_removed));
    MIC_TRY(mic_find_marker_cells(ctx, &n));
  }
  // main:255-268: marker density anomaly, projection
  MIC_TRY(mic_update_marker_rho(ctx));
  MIC_TRY(mic_project_markers_nodes_all2(ctx));
  // main:271-289: melting check
  MIC_TRY(mic_max_marker_T(ctx, &rep->max_T));
  if (rep->max_T > 9999.0) {  // TBREAK
    rep->stopped = 1;
    return MIC_OK;
  }
  // main:292-362: plasticity iterations
  double displacementdt = o->dtMax;
  int isYielding = 1, converged = 0, iPlastic = 0;
  const double gy = o->sub.gy;
  while ((o->firstStep && iPlastic < 1) || ((isYielding || !converged) && iPlastic < o->maxNumPlasticity)) {
    isYielding = 0;
    converged = 0;
    MIC_TRY(mic_check_plastic_yielding(ctx, displacementdt, &isYielding, elapsed_time));
    MIC_TRY(mic_limit_viscosity(ctx));
    MIC_TRY(mic_project_markers_nodes_all2(ctx));
    if (!o->staticVelocity || !ctx->sys[0].factored || !ctx->solution) {
      MIC_TRY(mic_form_vep_system(ctx, &o->sub, displacementdt, &rep->Kbond, &rep->Kcont));
      MIC_TRY(mic_linear_solve(ctx, 0));
    } else {  // main:315-317: the steady solution again, with the Kcont of its assembly
      rep->Kbond = ctx->sys[0].Kbond;
      rep->Kcont = ctx->sys[0].Kcont;
    }
    int fn = 0;
    MIC_TRY(mic_retrieve_solutions(ctx, nullptr, rep->Kcont, &fn));
    if (fn) return MIC_ERR_NAN;
    MIC_TRY(mic_nodal_stress_strain(ctx, displacementdt, gy));
    MIC_TRY(mic_update_marker_strain_pressure(ctx, displacementdt));
    MIC_TRY(mic_update_global_strain_rate_residual(ctx, iPlastic, &rep->residual));
    MIC_TRY(mic_check_convergence(ctx, 1e-16, 1e-1, iPlastic, &converged));
    const double lastdt = displacementdt;
    MIC_TRY(mic_limit_displacement_timestep(ctx, o->displacementStepLimit, &displacementdt));
    if (displacementdt != lastdt) converged = 0;
    ++iPlastic;
  }
  rep->plastic_iterations = iPlastic;
  rep->is_yielding = isYielding;
  rep->converged = converged;
  rep->displacement_dt = displacementdt;
  double dt = displacementdt;
  // main:369-376: sub-grid stress diffusion, stress update, heating
  if (ctx->opt.subgridStressDiffusivity > 0.0)
    MIC_TRY(mic_subgrid_stress_changes(ctx, displacementdt, ctx->opt.subgridStressDiffusivity));
  MIC_TRY(mic_update_marker_stress(ctx));
  if (!o->shearHeating)
    MIC_CUDA_TRY(cudaMemsetAsync(ctx->nodal[MIC_NF_HEATING], 0, sizeof(double) * ctx->P.NX * ctx->P.NY,
                                 ctx->stream));
  if (o->adiabaticHeating) MIC_TRY(mic_adiabatic_heating(ctx, o->sub.gy));
  // main:379-403: thermal solve, repeated with a shorter step for a too large change
  MIC_TRY(thermal_solve(ctx, *o, dt));
  double dTmax = 0.0;
  MIC_TRY(max_temp_change(ctx, &dTmax));
  if (dTmax > o->maxTempChange) {
    dt = dt * o->maxTempChange / dTmax;
    MIC_TRY(thermal_solve(ctx, *o, dt));
    rep->thermal_resolves = 1;
    MIC_TRY(max_temp_change(ctx, &dTmax));
  }
  rep->max_temp_change = dTmax;
  rep->dt = dt;
  // main:409, 435: sub-grid temperature changes with the new temperature, the diagnostics,
  // advection
  MIC_TRY(mic_subgrid_temperature_changes(ctx, dt));
  MIC_TRY(mic_nusselt_number(ctx, o->thermalBCBottomValue, o->sub.thermalBCTopValue, &rep->nusselt));
  MIC_TRY(mic_rms_velocity(ctx, &rep->vrms));
  MIC_TRY(mic_advect_markers_rk(ctx, dt));
  MIC_TRY(mic_max_abs_sxx(ctx, &rep->max_abs_sxx));
  MIC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return MIC_OK;
}

// Monte-Carlo members side by side.  fvmic2d's main runs its realisations one after another
// (the iMonte loop, main_subduction.c); here independent contexts step together, one host
// thread per member at a time, so that their sequential parts (the solver's panel chains, the
// host decisions between passes) overlap on the GPU instead of queueing behind each other.
extern "C" int mic_subduction_timestep_many(mic_ctx *const *ctxs, int n, const mic_timestep_options *options,
                                            const double *elapsed_time, mic_timestep_report *reports,
                                            int *codes, int max_threads) {
  if (!ctxs || n < 0 || !options || !reports) return MIC_ERR_ARG;
  for (int k = 0; k < n; ++k)
    if (!ctxs[k]) return MIC_ERR_ARG;
  int nt = max_threads > 0 ? max_threads : (int)std::thread::hardware_concurrency();
  nt = std::max(1, std::min(nt, n));
  std::atomic<int> next(0);
  std::vector<int> rc(n, MIC_OK);
  auto work = [&]() {
    for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1))
      rc[k] = mic_subduction_timestep(ctxs[k], &options[k], elapsed_time ? elapsed_time[k] : 0.0, &reports[k]);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
  int first = MIC_OK;
  for (int k = 0; k < n; ++k) {
    if (codes) codes[k] = rc[k];
    if (rc[k] && !first) first = rc[k];
  }
  return first;
}
