"""Benchmark: markers/s per step of the marker-in-cell transfer path on GB300.

Workload (default): the composite ice creep box, 1025 x 1025 nodes, 16,777,216 markers, material
law 7 (the Goldsby-Kohlstedt law of viscosity.c:106-179 inverted per marker), FP64 -- the
configuration the metric is quoted on.  A step is one pass of fvmic2d's marker path in
main_subduction.c order (bin + stable sort, density update, projectMarkersNodesAll2, max T,
checkPlasticYielding, limitViscosity, projectMarkersNodesAll2, updateMarkerStrainPressure,
updateGlobalStrainRateResidual, subgridStressChanges, updateMarkerStress,
subgridTemperatureChanges, advectMarkersRK, max |sxx|), with the host Stokes/thermal solves
outside the timed region; their nodal outputs are synthetic inputs held on the device.  The
law-7 stress solve runs two ways on the same context: the plain exact solve, and the trained
surrogate with the hidden layer on the tensor cores, FP64 polish and exact fallback.  `value` is
the surrogate path's markers/s; the plain path's sits beside it under `plain`.  The
visco-elasto-plastic box (1025 x 257 nodes, 4,194,304 markers) and the ensembles ride along as
extra legs.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]

One JSON line on rank 0.  Under torchrun (N > 1) every rank runs an independent replica on its
own GPU (the path shards only across independent problems); value = all markers processed /
max-over-ranks time.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "markers/s per step (project+advect+rheology), plain vs surrogate @1e-6 rel err"
WORKLOAD_DESC = {
    "ice_creep_box": ("ice_creep_box: 1025x1025 uniform nodes, 16 markers/cell, 16,777,216 markers, composite ice "
                      "creep (law 7) with per-marker log10 edot ~ U[-18,-10] 1/s, T ~ U[100,273] K, log10 grain size "
                      "~ U[-4,-1] m, P ~ U[0,1e8] Pa (SplitMix64 seed 3); MLP 4->64->64->1, BF16 hidden layer on the "
                      "tensor cores with FP32 accumulation, FP64 polish to |rate/edot - 1| <= 1e-7, exact fallback; FP64"),
    "vep_slab_box": ("vep_slab_box: 1025x257 staggered grid (2x refined top 20%), 16 markers/cell, "
                     "4,194,304 markers, two materials, Mohr-Coulomb yield, FP64"),
    "convection_box": ("convection_box: unit-square thermal convection, viscosity exp(-ln(1000) T), free slip, "
                       "T0 = 1 - y + 0.01 cos(pi x) sin(pi y), 64x64 cells (65x65 nodes), 16 jittered markers/cell, "
                       "65,536 markers, 10 steps, FP64"),
}
CONVECTION_STEPS = 10  # the convection configuration's step count
# the bounded sample of each workload that the host-core baseline steps: the same generator and
# per-marker distributions on a smaller grid
CPU_SAMPLE = {"ice_creep_box": "ice_creep_box_sample", "vep_slab_box": "vep_slab_box_sample",
              "ice_creep_box_4m": "ice_creep_box_sample", "vep_slab_box_1m": "vep_slab_box_sample"}
CPU_SAMPLE_DESC = {"ice_creep_box_sample": "129x129 nodes, 262,144 markers",
                   "vep_slab_box_sample": "257x65 nodes, 262,144 markers"}
# law-7 settings of the timed paths: exact solve to |rate/edot - 1| <= 2e-14; surrogate polish to
# 1e-7 (stress within 1e-7 of the exact root) in at most 3 steps, else the exact solve
CREEP_TOL, CREEP_MAXIT, POLISH_ITERS, POLISH_TOL = 2e-14, 60, 3, 1e-7

# Host-solve outputs that cross the boundary each step in the drop-in model (markers stay
# resident on the device): nodal inputs up, projected nodal fields down.
E2E_UP = ["vx", "vy", "p", "edotxx", "edotyy", "edotxy", "wxy", "soxx", "soyy", "soxy", "dsxx", "dsyy", "dsxy",
          "thisT"]
E2E_DOWN = ["rho", "etaN", "etaS", "kThermal", "lastT", "Cp", "soxx", "soyy", "soxy"]

# Algorithmic bytes per marker of the whole step (compulsory marker-state traffic of the five
# dependency-forced passes) and per node (44 nodal-array touches of 8 bytes).
STEP_BYTES_PER_MARKER = 436
STEP_BYTES_PER_NODE = 352

# Per-kernel algorithmic bytes: each kernel's own inputs read once and outputs written once
# (marker columns per marker, nodal arrays per node).  Indexing and scratch re-reads are not
# credited.
KERNEL_BYTES = {
    # X, Y read; cellX, cellY, key, cpu written
    "k_find_cells": (16 + 16, 0),
    # cellX, flags, 4 offsets, eta, rho, T, sxx, syy, sxy, Mat read; 12 nodal fields written
    "k_project_all2": (4 + 4 + 32 + 48 + 4, 96),
    # cellX, cellY, X, Y, s3, e3, Eii read; X, Y, VX, VY, wxy, s3, Eii written; vx, vy, wxy read
    "k_advect": (8 + 16 + 24 + 24 + 8 + 16 + 16 + 8 + 24 + 8, 24),
    # cellX, cellY, flags, 4 offsets, X, Y, eta, mu read; p, e3, wxy, srr written; 10 nodal read
    "k_strain_pressure": (8 + 4 + 32 + 16 + 16 + 8 + 24 + 8 + 8, 80),
    # plastic materials: cellX, Mat, T, p, Eii, e3, eta, mu, s3 read; eta, mu, s3 written
    "k_yield": (4 + 4 + 8 + 8 + 8 + 24 + 16 + 24 + 40, 0),
    # all 29 marker columns read and written
    "k_reorder": (2 * (23 * 8 + 6 * 4) + 4, 0),
}


# The law-7 pass of the ice workload (no plastic yield: the visco-elastic forecast and stresses are
# not read): cellX, Mat, T, p, e3, eta, mu and the grain factor read; eta, mu written
KERNEL_BYTES_LAW7 = {k: (4 + 4 + 8 + 8 + 24 + 16 + 8 + 16, 0) for k in ("k_yield", "k_yield_tc",
                                                                      "k_yield_surrogate_fp32")}


# DRAM bytes per marker of one launch from an ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum) of the 4,194,304-marker ice box (the first step of each mode), scaled to a
# full launch by markers processed (profiles/fp64_mix_ice_creep_box_4m.md).  The advection reads
# the algorithmic bytes plus the 32 B/marker of stored offsets its first RK4 stage loads instead
# of forming them.
KERNEL_TRAFFIC_PER_MARKER = {"k_advect": 792.6e6 / 4194304, "k_yield_tc": 424.5e6 / 4194304,
                             "k_yield": 421.5e6 / 4194304}
# FP64 work per marker from the same captures (DFMA and DADD + DMUL thread instructions per
# marker): flops with a DFMA counted twice, and the FP64 arithmetic instructions.  The exact law-7
# pass (k_yield) is bound by the FP64 pipe, which issues 2 FP64 instructions per SM per clock on
# GB300; the advection mostly, with its interpolations in double-float arithmetic on the FP32
# pipe; the tensor-core surrogate pass runs its polish in double-float arithmetic and is bound by
# instruction issue (KERNEL_INST_PER_MARKER: every thread instruction, all pipes).
_FP64_PER_MARKER = {"k_advect": (14.0, 45.0), "k_yield_tc": (5.0, 10.0), "k_yield": (65.7, 130.6)}
KERNEL_FP64_FLOPS_PER_MARKER = {k: 2 * f + u for k, (f, u) in _FP64_PER_MARKER.items()}
KERNEL_FP64_INST_PER_MARKER = {k: f + u for k, (f, u) in _FP64_PER_MARKER.items()}
KERNEL_INST_PER_MARKER = {"k_advect": 3070.0, "k_yield_tc": 4066.0, "k_yield": 2885.0}
ISSUE_PEAK_GINST = 4 * 32 * 152 * 2.07  # thread instructions per second, in G (4 warp issues/SM/clk)
FP64_PEAK_TFLOPS = 2 * 2 * 152 * 2.07e9 / 1e12  # 2 DFMA/SM/clk x 2 flops x 152 SMs x 2.07 GHz
FP64_PEAK_GINST = 2 * 152 * 2.07  # FP64 instructions per second, in G


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ice_creep_box")
    ap.add_argument("--no-legs", action="store_true", help="main workload only (no VEP, ensemble, systems legs)")
    ap.add_argument("--no-vep", action="store_true", help="skip the visco-elasto-plastic box leg")
    ap.add_argument("--no-convection", action="store_true", help="skip the 64x64 convection box leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble legs")
    ap.add_argument("--no-systems", action="store_true", help="skip the linear-systems / whole-time-step leg")
    ap.add_argument("--only-systems", action="store_true",
                    help="run only the linear-systems / whole-time-step leg and print it (for profiling the solver)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (no mic_autotune)")
    ap.add_argument("--cpu-cores", type=int, default=0, help="host processes for the CPU legs (0 = all)")
    return ap.parse_args()


def make_workload(name):
    from fvmic2d_gb300 import workloads as W

    return W.WORKLOADS[name]()


# ---------------------------------------------------------------------------------------
# CPU legs: the CPU restatement of the reference path (oracle/liboracle.so, gcc -O2
# -ffp-contract=off), one process per core, each stepping its own replica of a bounded sample of
# the workload (spawned before any GPU work).


def _cpu_worker(args):
    name, steps, warmup, barrier = args
    sys.path.insert(0, ROOT)
    from oracle import oraclepy

    wl = make_workload(name)
    P = oraclepy.OracleProblem(wl)
    if getattr(wl, "grain_size", None) is not None:
        P.set_grain_size(wl.grain_size)
    for _ in range(warmup):
        P.step(wl.dt, wl.dt_thermal)
    barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        e, _ = P.step(wl.dt, wl.dt_thermal)
        if e:
            raise RuntimeError("oracle step failed with %d" % e)
    t1 = time.perf_counter()
    return len(wl.markers), t1 - t0


def cpu_throughput(name, cores, steps, warmup):
    """Aggregate markers/s of `cores` concurrent single-threaded replicas."""
    from oracle import build as obuild

    obuild.build_oracle()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        barrier = man.Barrier(cores)
        with ctx.Pool(cores) as pool:
            res = pool.map(_cpu_worker, [(name, steps, warmup, barrier)] * cores)
    n = sum(r[0] for r in res) * steps
    t = max(r[1] for r in res)
    return n / t, t / steps * 1e3


def host_cores(requested):
    n = os.cpu_count() or 1
    return max(1, min(n, requested)) if requested else n


def cpu_sample(name):
    """the workload the host-core baseline steps for `name` (itself when it has no smaller sample)"""
    return CPU_SAMPLE.get(name, name)


def cpu_sample_text(name, cores, steps, rate1=None, ms1=None):
    sample = cpu_sample(name)
    what = ("%s (%s; the full workload's generator and per-marker distributions on a smaller grid)"
            % (sample, CPU_SAMPLE_DESC[sample]) if sample in CPU_SAMPLE_DESC else "the full workload " + sample)
    txt = ("%d step(s) per replica of %s, %d concurrent single-threaded replicas; CPU restatement of the reference "
           "path, gcc -O2 -ffp-contract=off (the reference tree is not on this host)" % (steps, what, cores))
    if rate1 is not None:
        txt += "; single replica: %.4g markers/s, %.0f ms/step" % (rate1, ms1)
    return txt


# ---------------------------------------------------------------------------------------
# clocks during the timed region


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    p = [s.strip() for s in line.split(",")]
                    if len(p) >= 9:
                        rows.append(p)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = [s for s in sm if s >= 0.5 * (max(sm) if sm else 0)]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------------------


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def base_config(wl, name, world):
    state = len(wl.markers) * 208
    l2 = ("inputs larger than L2 (marker state %.2f GB per replica)" % (state / 1e9) if state > 129e6 else
          "inputs smaller than L2 (marker state %.1f MB): L2-resident between steps, no flush" % (state / 1e6))
    return {"workload": WORKLOAD_DESC.get(name, name),
            "markers_per_replica": int(len(wl.markers)), "nodes": [wl.grid.NX, wl.grid.NY],
            "parallelism": "replicas x%d (independent problems, no collective)" % world,
            "l2": l2,
            "timed": "bin+sort, rho, project x2, max T, yield (law-7 stress solve), limit, strain/pressure, residual, "
                     "subgrid stress, stress update, subgrid T, RK4 advection, max |sxx|; host solves excluded"}


def run_reference_arm(args):
    """The reference's CPU path on the host cores: the C restatement (pinned bit for bit to the
    reference's own sources, which are not on this host), one single-threaded replica per core,
    each stepping a bounded sample of the workload for warmup + steps steps."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    cores = host_cores(args.cpu_cores)
    rate, ms = cpu_throughput(cpu_sample(args.workload), cores, args.steps, args.warmup)
    wl = make_workload(args.workload)
    line = {"metric": METRIC, "value": rate, "unit": "markers/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)",
            "config": base_config(wl, args.workload, 1), "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": "markers/s", "cores": cores, "kind": "port",
                             "sample": cpu_sample_text(args.workload, cores, args.steps)},
            "e2e": {"value": rate, "unit": "markers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return float(json.load(open(path))["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback"


def timed_steps(G, wl, args, pg, label):
    """warmup, launch shapes, then `steps` steps between CUDA events on the context's stream, and
    the same steps again with an event pair around every launch for the per-kernel durations"""
    import torch

    from fvmic2d_gb300 import gpu

    L, h = G.L, G.h
    stream = torch.cuda.ExternalStream(G.stream(), device=G.device)
    sub = 1 if wl.options.subgridStressDiffusivity > 0 else 0

    def step():
        e = L.mic_step(h, wl.dt, wl.dt_thermal, sub, None)
        if e:
            raise gpu.MicError(e, "mic_step")

    for _ in range(args.warmup):
        step()
    G.synchronize()
    # launch shapes measured on this workload (state restored afterwards; outside the timing)
    tuning = G.autotune(wl.dt, wl.dt_thermal, subgrid_stress=sub, steps=2) if not args.no_autotune else None
    launches0 = G.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(G.device) as clk:
        torch.cuda.synchronize()
        barrier(pg)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        barrier(pg)
    launches = G.launch_count() - launches0
    ms_total = ev0.elapsed_time(ev1)
    G.profile_enable(max(64, 64 * args.steps))  # room for every launch (44 per step)
    for _ in range(args.steps):
        step()
    G.synchronize()
    prof = G.profile_read()
    G.profile_enable(0)
    recorded = sum(v[1] for v in prof.values())
    if recorded != launches:  # a truncated record would understate every per-step figure
        raise RuntimeError("per-launch profile holds %d of %d launches (%s)" % (recorded, launches, label))
    n = G.n
    t_max = max_over_ranks(pg, ms_total)
    value = sum_over_ranks(pg, float(n * args.steps)) / (t_max * 1e-3)
    out = {"value": value, "unit": "markers/s", "ms_per_step": t_max / args.steps, "gpu_launches": launches,
           "launch_tuning": tuning, "clocks": clk.summary()}
    return out, prof


def roofline(prof, n, nodes, steps, hbm_peak, peak_src, law7=False):
    """HBM roofline of the step's dominant kernel (live CUDA-event duration), with its FP64 issue
    rate where ncu measured its FP64 instructions per marker"""
    kern = sorted(prof.items(), key=lambda kv: -kv[1][0])
    # a kernel on the second stream (the first projection's partial sums) overlaps the yield pass:
    # its event span is not its own cost, so the dominant kernel is taken among the main stream's
    main = [kv for kv in kern if not kv[0].startswith(("k_partials_basic<first>", "k_partials_centre<scalar>",
                                                        "k_combine_scalar<-1>", "k_residual_weight"))]
    top_name, (top_ms, top_cnt) = (main or kern)[0]
    table = dict(KERNEL_BYTES, **(KERNEL_BYTES_LAW7 if law7 else {}))
    per_marker, per_node = table.get(top_name, (0, 0))
    algo = per_marker * n + per_node * nodes
    dur = top_ms / max(top_cnt, 1)
    achieved = algo / (dur * 1e-3) / 1e9
    prof_total = sum(v[0] for v in prof.values())
    roof = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak,
            "traffic": (KERNEL_TRAFFIC_PER_MARKER[top_name] * n if top_name in KERNEL_TRAFFIC_PER_MARKER else None),
            "traffic_note": "ncu dram bytes of the 4,194,304-marker capture of the same kernel, scaled by markers "
                            "processed",
            "peak_source": peak_src, "algorithmic_bytes_per_launch": algo, "ms_per_launch": dur}
    fp64 = None
    if top_name in KERNEL_FP64_INST_PER_MARKER and (law7 or not top_name.startswith("k_yield")):
        ipm = KERNEL_FP64_INST_PER_MARKER[top_name]
        fpm = KERNEL_FP64_FLOPS_PER_MARKER[top_name]
        fp64 = {"kernel": top_name, "flops_per_marker": fpm, "achieved": fpm * n / (dur * 1e-3) / 1e12,
                "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": fpm * n / (dur * 1e-3) / 1e12 / FP64_PEAK_TFLOPS,
                "inst_per_marker": ipm, "issue_frac": ipm * n / (dur * 1e-3) / 1e9 / FP64_PEAK_GINST,
                "note": "FP64 pipe, 2 FP64 instructions/SM/clk; flops and instructions per marker from ncu; "
                        "issue_frac = FP64 instructions issued / peak"}
        if top_name in KERNEL_INST_PER_MARKER:
            ins = KERNEL_INST_PER_MARKER[top_name]
            fp64["all_inst_per_marker"] = ins
            fp64["all_issue_frac"] = ins * n / (dur * 1e-3) / 1e9 / ISSUE_PEAK_GINST
            fp64["all_issue_note"] = ("every thread instruction (all pipes) from ncu against 4 warp instructions "
                                      "per SM per clock: the bound of a pass whose FP64 work moved to the FP32 pipe")
    shares = {k: round(v[0] / prof_total, 4) for k, v in kern[:12]}
    per_step = {k: round(v[0] / steps, 4) for k, v in kern[:12]}
    return roof, fp64, shares, per_step


def e2e_run(G, wl, steps, pg):
    """the same step end to end through the C ABI with pinned host buffers: the host-solve nodal
    fields up and the projected nodal fields down every step"""
    import ctypes

    import numpy as np

    from fvmic2d_gb300.mic_types import NF

    L, h = G.L, G.h
    nodes = wl.grid.NX * wl.grid.NY
    n = G.n
    sub = 1 if wl.options.subgridStressDiffusivity > 0 else 0

    def pinned(nbytes):
        p = ctypes.c_void_p()
        assert L.mic_host_alloc(ctypes.byref(p), nbytes) == 0
        return p

    up_bufs, down_bufs = [], []
    for name in E2E_UP:
        p = pinned(nodes * 8)
        a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(nodes,))
        a[:] = np.asarray(wl.nodal[name], dtype=np.float64).ravel()
        up_bufs.append((NF[name], p, a))
    for name in E2E_DOWN:
        p = pinned(nodes * 8)
        a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(nodes,))
        down_bufs.append((NF[name], p, a))
    res = ctypes.c_double(0.0)
    up_f = (ctypes.c_int * len(up_bufs))(*[fid for fid, _, _ in up_bufs])
    up_p = (ctypes.c_void_p * len(up_bufs))(*[p.value for _, p, _ in up_bufs])
    dn_f = (ctypes.c_int * len(down_bufs))(*[fid for fid, _, _ in down_bufs])
    dn_p = (ctypes.c_void_p * len(down_bufs))(*[p.value for _, p, _ in down_bufs])

    def e2e_step():
        assert L.mic_nodal_upload_many(h, up_f, up_p, len(up_bufs)) == 0
        assert L.mic_step(h, wl.dt, wl.dt_thermal, sub, ctypes.byref(res)) == 0
        assert L.mic_nodal_download_many(h, dn_f, dn_p, len(down_bufs)) == 0

    e2e_steps = max(3, min(steps, 50))
    e2e_step()
    G.synchronize()
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    G.synchronize()
    t_e2e = max_over_ranks(pg, time.perf_counter() - t0)
    value = sum_over_ranks(pg, float(n * e2e_steps)) / t_e2e
    for _, p, _ in up_bufs + down_bufs:
        L.mic_host_free(p)
    return {"value": value, "unit": "markers/s", "h2d_bytes_per_step": len(E2E_UP) * nodes * 8,
            "d2h_bytes_per_step": len(E2E_DOWN) * nodes * 8 + 8,
            "model": "markers resident on the device; host-solve nodal fields up and projected nodal fields down "
                     "every step from/to pinned host buffers through mic_nodal_upload_many / mic_step / "
                     "mic_nodal_download_many"}


def surrogate_error_in_step(G, wl):
    """The surrogate's stress error on the stepped workload, judged by the exact solve: the
    law-7 viscosity of every marker from the same marker state by checkPlasticYielding with the
    exact solve and with the surrogate (eta = s* / (2 edot), so the relative viscosity error is the
    relative stress error; the ice has no plastic yield, so the pass leaves everything but eta and
    mu as it found it)"""
    import numpy as np

    G.creep_configure(mode=0, tol=CREEP_TOL, maxit=CREEP_MAXIT, polish_iters=POLISH_ITERS, polish_tol=POLISH_TOL)
    G.checkPlasticYielding(wl.dt)
    eta0 = G.markers["eta"]
    G.creep_configure(mode=2, tol=CREEP_TOL, maxit=CREEP_MAXIT, polish_iters=POLISH_ITERS, polish_tol=POLISH_TOL)
    G.checkPlasticYielding(wl.dt)
    st = G.creep_stats()
    eta2 = G.markers["eta"]
    ok = np.isfinite(eta0) & (eta0 > 0)
    rel = np.abs(eta2[ok] / eta0[ok] - 1.0)
    return {"max": float(rel.max()), "median": float(np.median(rel)), "markers": int(ok.sum()),
            "fallbacks": st["fallbacks"], "max_residual": st["max_residual"], "tc_timeouts": st["tc_timeouts"],
            "sample": "every marker of the workload after the timed steps: surrogate vs exact solve from the same "
                      "state (one checkPlasticYielding pass each)"}


def surrogate_error_batch(G):
    """the same comparison on 1,048,576 fresh samples of the workload's input distribution"""
    import numpy as np

    from fvmic2d_gb300 import workloads as W

    m = 1 << 20
    u = W.splitmix64_uniform(11, 4 * m)
    edot, T, d, P = 10 ** (-18 + 8 * u[0::4]), 100 + 173 * u[1::4], 10 ** (-4 + 3 * u[2::4]), 1e8 * u[3::4]
    G.creep_configure(mode=0, tol=CREEP_TOL, maxit=CREEP_MAXIT, polish_iters=POLISH_ITERS, polish_tol=POLISH_TOL)
    s0, it0, _, _ = G.creep_solve(edot, T, d, P, mode=0)
    s2, it2, _, fb = G.creep_solve(edot, T, d, P, mode=2)
    rel = np.abs(s2 / s0 - 1.0)
    return {"max": float(rel.max()), "median": float(np.median(rel)), "fallbacks": int(fb.sum()),
            "iters_exact": float(it0.mean()), "iters_surrogate": float(it2.mean()),
            "sample": "%d solves, tensor-core surrogate vs exact" % m}


def measure_workload(args, name, local, pg, world, cpu=None, with_e2e=True, with_density=True):
    """One marker-path workload timed on one context: for law 7 the exact solve ("plain") and the
    tensor-core surrogate, the surrogate being the headline; otherwise the plain path."""
    import torch

    from fvmic2d_gb300 import gpu

    wl = make_workload(name)
    G = gpu.MicProblem(wl, device=local)
    G.device = local
    law7 = getattr(wl, "grain_size", None) is not None
    out = {}
    if law7:
        G.set_grain_size(wl.grain_size)
        t0 = time.perf_counter()
        hist = G.creep_train()
        torch.cuda.synchronize()
        out["train"] = {"seconds": round(time.perf_counter() - t0, 3), "loss_final": float(hist[-200:].mean()),
                        "loss_first": float(hist[:50].mean()),
                        "note": "surrogate trained on the GPU (2,097,152 exact solves, 10,000 Adam steps), "
                                "outside the timed region"}
    modes = [("plain", 0), ("surrogate_tc", 2)] if law7 else [("plain", 0)]
    hbm_peak, peak_src = read_peaks()
    n, nodes = G.n, wl.grid.NX * wl.grid.NY
    for label, mode in modes:
        if law7:
            G.creep_configure(mode=mode, tol=CREEP_TOL, maxit=CREEP_MAXIT, polish_iters=POLISH_ITERS,
                              polish_tol=POLISH_TOL)
        rec, prof = timed_steps(G, wl, args, pg, label)
        roof, fp64, shares, per_step = roofline(prof, n, nodes, args.steps, hbm_peak, peak_src, law7)
        rec.update({"roofline": roof, "fp64_roofline": fp64, "kernel_share": shares, "kernel_ms_per_step": per_step})
        if law7:
            st = G.creep_stats()
            yk = [k for k in prof if k.startswith("k_yield")]
            rec.update({"yield_kernel": yk[0] if yk else None,
                        "yield_ms_per_step": prof[yk[0]][0] / args.steps if yk else None,
                        "newton_iters_per_marker": st["iterations"] / max(st["markers"], 1),
                        "fallbacks_per_step": st["fallbacks"], "tc_timeouts": st["tc_timeouts"],
                        "max_residual": st["max_residual"]})
        step_bytes = STEP_BYTES_PER_MARKER * n + STEP_BYTES_PER_NODE * nodes + (8 * n if law7 else 0)
        gbs = step_bytes / (rec["ms_per_step"] * 1e-3) / 1e9
        rec["step_roofline"] = {"algorithmic_bytes_per_step": step_bytes, "achieved_gbs": gbs, "frac": gbs / hbm_peak}
        out[label] = rec
    head = out["surrogate_tc" if law7 else "plain"]
    if law7:
        out["speedup_surrogate_vs_plain"] = head["value"] / out["plain"]["value"]
        out["yield_speedup_surrogate_vs_plain"] = out["plain"]["yield_ms_per_step"] / head["yield_ms_per_step"]
    if with_e2e:
        out["e2e"] = e2e_run(G, wl, args.steps, pg)  # in the headline mode (the last configured)
    if law7:
        out["stress_rel_err"] = surrogate_error_in_step(G, wl)
        out["stress_rel_err_batch"] = surrogate_error_batch(G)
    if with_density and int(os.environ.get("RANK", "0")) == 0:
        # checkMarkerDensity (called every step by the reference) after the steps moved the
        # markers, with the reference's default bounds (1 and 100 per quarter cell)
        from fvmic2d_gb300.mic_types import DensityOptions

        dopt = DensityOptions(NMX=4, NMY=4, minMarkers=1, maxMarkers=100)
        G.synchronize()
        t0 = time.perf_counter()
        reps = 5
        tot_add = tot_rem = 0
        for _ in range(reps):
            a, r_ = G.checkMarkerDensity(dopt)
            tot_add += a
            tot_rem += r_
        out["density_control"] = {"ms_per_call": (time.perf_counter() - t0) * 1e3 / reps, "markers_added": tot_add,
                                  "markers_removed": tot_rem, "calls": reps,
                                  "note": "host wall time per call, including its host synchronisations"}
    out["config"] = base_config(wl, name, world)
    if cpu is not None:
        out["cpu_baseline"] = cpu
    G.close()
    return out, head


def run_ours(args):
    world, rank, local, pg = dist_setup(args)
    if args.only_systems:
        if rank == 0:
            import torch

            torch.cuda.set_device(local)
            print(json.dumps({"systems": systems_leg(args, local)}), flush=True)
        return
    cpu = cpu_vep = cpu_conv = None
    legs = not args.no_legs
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # bounded samples: one step per replica on all host cores, and on one core, spawned before
        # any GPU work
        cores = host_cores(args.cpu_cores)
        rate, ms = cpu_throughput(cpu_sample(args.workload), cores, 1, 0)
        rate1, ms1 = cpu_throughput(cpu_sample(args.workload), 1, 1, 0)
        cpu = {"value": rate, "unit": "markers/s", "cores": cores, "kind": "port",
               "sample": cpu_sample_text(args.workload, cores, 1, rate1, ms1), "value_1core": rate1}
        if legs and not args.no_vep and args.workload != "vep_slab_box":
            rate, ms = cpu_throughput(cpu_sample("vep_slab_box"), cores, 1, 0)
            rate1, ms1 = cpu_throughput(cpu_sample("vep_slab_box"), 1, 1, 0)
            cpu_vep = {"value": rate, "unit": "markers/s", "cores": cores, "kind": "port",
                       "sample": cpu_sample_text("vep_slab_box", cores, 1, rate1, ms1), "value_1core": rate1}
        if legs and not args.no_convection:
            # the whole configuration (65,536 markers, 10 steps) on the host cores
            rate, ms = cpu_throughput("convection_box", cores, CONVECTION_STEPS, 0)
            rate1, ms1 = cpu_throughput("convection_box", 1, CONVECTION_STEPS, 0)
            cpu_conv = {"value": rate, "unit": "markers/s", "cores": cores, "kind": "port",
                        "sample": cpu_sample_text("convection_box", cores, CONVECTION_STEPS, rate1, ms1),
                        "value_1core": rate1}
    import torch

    torch.cuda.set_device(local)
    main, head = measure_workload(args, args.workload, local, pg, world)
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": head["value"], "unit": "markers/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)",
        "config": main.pop("config"),
        "clocks": head["clocks"],
        "e2e": main.pop("e2e"),
        "gpu_launches": head["gpu_launches"],
        "roofline": head["roofline"],
        "fp64_roofline": head["fp64_roofline"],
        "step_roofline": head["step_roofline"],
        "kernel_share": head["kernel_share"],
        "kernel_ms_per_step": head["kernel_ms_per_step"],
    }
    if "surrogate_tc" in main:
        line["config"]["path"] = "surrogate_tc (value); plain exact solve under plain"
        line["plain"] = {k: main["plain"][k] for k in ("value", "unit", "ms_per_step", "yield_kernel",
                                                       "yield_ms_per_step", "newton_iters_per_marker",
                                                       "fallbacks_per_step", "roofline", "fp64_roofline",
                                                       "kernel_ms_per_step", "clocks")}
        line["surrogate"] = {k: head[k] for k in ("yield_kernel", "yield_ms_per_step", "newton_iters_per_marker",
                                                  "fallbacks_per_step", "tc_timeouts", "max_residual")}
        for k in ("speedup_surrogate_vs_plain", "yield_speedup_surrogate_vs_plain", "stress_rel_err",
                  "stress_rel_err_batch", "train"):
            line[k] = main[k]
    line["density_control"] = main.get("density_control")
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if legs and not args.no_vep and args.workload != "vep_slab_box":
        vep, vhead = measure_workload(args, "vep_slab_box", local, None, 1, cpu=cpu_vep, with_density=False)
        vep["plain"].pop("launch_tuning", None)
        line["vep_slab_box"] = vep
    if legs and not args.no_convection:
        cargs = argparse.Namespace(**vars(args))
        cargs.steps, cargs.warmup = CONVECTION_STEPS, max(3, min(args.warmup, CONVECTION_STEPS))
        conv, _ = measure_workload(cargs, "convection_box", local, None, 1, cpu=cpu_conv, with_density=False)
        conv["plain"].pop("launch_tuning", None)
        line["convection_box"] = conv
    if legs and not args.no_ensemble:
        line["ensemble"] = ensemble_leg(args, local)
        line["ice_ensemble"] = ice_ensemble_leg(args, local)
    if legs and not args.no_systems:
        line["systems"] = systems_leg(args, local)
    print(json.dumps(line), flush=True)


ENSEMBLE_STEPS = 50  # the batching configurations' step count


def _time_ensemble(E, es, dts, steps, graph):
    """ms per ensemble step over `steps` steps (after three untimed ones), CUDA events on the
    ensemble stream, and kernels launched per step"""
    import torch

    for _ in range(3):
        E.step(dts, dts, 1, graph)
    E.synchronize()
    l0, _ = E.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(es)
    for _ in range(steps):
        E.step(dts, dts, 1, graph)
    ev1.record(es)
    ev1.synchronize()
    l1, _ = E.launch_count()
    return ev0.elapsed_time(ev1) / steps, (l1 - l0) / steps


def ensemble_leg(args, local):
    """Ensemble of independent convection runs (64 members, mixed grids): the same steps issued
    one member at a time (each step waiting for the host, as a plain loop over problems does);
    per-member (every member's own kernels on its stream) and batched (one kernel per marker pass
    over all members), each on streams and as one captured CUDA graph per ensemble step; then the
    schedule mic_ensemble_autotune picks."""
    import numpy as np
    import torch

    from fvmic2d_gb300 import gpu
    from fvmic2d_gb300 import workloads as W

    wls = W.convection_ensemble()
    members = []
    for wl in wls:
        P = gpu.MicProblem(wl, device=local, capacity=wl.capacity)
        gpu.initialize_markers(P, *wl.nm, seed=wl.seed)
        members.append(P)
    n_total = sum(P.n for P in members)
    E = gpu.MicEnsemble(members)
    es = torch.cuda.ExternalStream(E.stream(), device=local)
    dts = np.array([wl.dt for wl in wls])
    steps = ENSEMBLE_STEPS
    out = {"workload": "convection_ensemble: 64 independent thermal-convection runs, square grids drawn from "
                       "{64^2,128^2,256^2,512^2} cells, 9/16/25 markers per cell, Ra log-uniform 1e4-1e7, viscosity "
                       "contrast log-uniform 1e1-1e5 (SplitMix64 seed 4); markers laid out on the device by "
                       "resetMarkers + distributeMarkersUniformInDomain",
           "members": len(members), "markers": int(n_total), "steps": steps}
    # one member at a time, host waiting on each (the residual read of mic_step)
    seq_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        for P, dt in zip(members, dts):
            P.step(dt, dt, True)
    t0 = time.perf_counter()
    for _ in range(seq_steps):
        for P, dt in zip(members, dts):
            P.step(dt, dt, True)
    ms = (time.perf_counter() - t0) * 1e3 / seq_steps
    out["sequential"] = {"value": n_total / (ms * 1e-3), "unit": "markers/s", "ms_per_step": ms,
                         "steps": seq_steps}
    # per-member kernels; batched marker passes in the default four groups and in one group
    for mode, groups in (("per_member", 0), ("batched", 4), ("batched_1group", 1)):
        E.set_schedule(groups=groups, chunked=2)
        for label, graph in (("streams", False), ("graph", True)):
            ms, kps = _time_ensemble(E, es, dts, steps, graph)
            out[mode + "_" + label] = {"value": n_total / (ms * 1e-3), "unit": "markers/s", "ms_per_step": ms,
                                       "kernels_per_step": kps}
    for mode in ("batched", "batched_1group"):
        out["speedup_%s_vs_per_member_graph" % mode] = (out[mode + "_graph"]["value"] /
                                                         out["per_member_graph"]["value"])
    out["speedup_graph_vs_sequential"] = out["batched_graph"]["value"] / out["sequential"]["value"]
    # members' launch shapes, the member order and the batching schedule from mic_ensemble_autotune
    # (state restored by it), then the captured steps timed again
    E.synchronize()
    t_tune = time.perf_counter()
    order = E.autotune(dts, dts, 1, steps=2)
    t_tune = time.perf_counter() - t_tune
    sizes = [members[i].n for i in order]
    ms, kps = _time_ensemble(E, es, dts, steps, True)
    out["graph_tuned"] = {"value": n_total / (ms * 1e-3), "unit": "markers/s", "ms_per_step": ms,
                          "kernels_per_step": kps, "tune_seconds": t_tune, "schedule": E.schedule(),
                          "order": ("largest first" if sizes == sorted(sizes, reverse=True) else
                                    "smallest first" if sizes == sorted(sizes) else "as given"),
                          "member_blocks_k_advect": sorted(set(P.tuning()["k_advect"] for P in members))}
    E.close()
    for P in members:
        P.close()
    return out


def ice_ensemble_leg(args, local):
    """Mixed ensemble with the learned closure: 256 independent ice-creep VEP boxes (grids from
    128^2 to 1024 x 256 cells, 16 markers per cell, law 7 with per-marker grain sizes,
    Drucker-Prager yield), 50 captured-graph steps with the exact creep solve and with the
    tensor-core surrogate (one network trained once, shared by all members), each per-member and
    batched (four batch groups, the default, and one group)."""
    import torch

    from fvmic2d_gb300 import gpu
    from fvmic2d_gb300 import workloads as W

    wls = W.ice_ensemble()
    members = []
    for wl in wls:
        P = gpu.MicProblem(wl, device=local, capacity=wl.capacity)
        gpu.initialize_markers(P, *wl.nm, seed=wl.seed)
        P.set_grain_size(W.ice_grain_sizes(P.n, wl.seed))
        members.append(P)
    n_total = sum(P.n for P in members)
    t0 = time.perf_counter()
    members[0].creep_train()
    train_s = time.perf_counter() - t0
    params = members[0].creep_params()
    for P in members[1:]:
        P.creep_set_params(params)
    E = gpu.MicEnsemble(members)
    es = torch.cuda.ExternalStream(E.stream(), device=local)
    dts = [wl.dt for wl in wls]
    steps = ENSEMBLE_STEPS
    out = {"workload": "ice_ensemble: 256 independent ice-creep VEP boxes (law 7, Drucker-Prager yield, "
                       "shear modulus 3.5 GPa), grids drawn from {128^2, 256x64, 128x256, 192^2, 1024x256} cells "
                       "(SplitMix64 seed 5), 16 markers per cell, per-marker log10 grain size ~ U[-4,-1] m",
           "members": len(members), "markers": int(n_total), "steps": steps, "train_seconds": round(train_s, 3)}
    for label, mode in (("plain", 0), ("surrogate_tc", 2)):
        for P in members:
            P.creep_configure(mode=mode, tol=2e-14, maxit=60, polish_iters=3, polish_tol=1e-7)
        for sched, groups in (("per_member", 0), ("batched", 4), ("batched_1group", 1)):
            E.set_schedule(groups=groups, chunked=2)
            ms, kps = _time_ensemble(E, es, dts, steps, True)
            st = [P.creep_stats() for P in members]
            mk = sum(x["markers"] for x in st)
            out[label + "_" + sched] = {"value": n_total / (ms * 1e-3), "unit": "markers/s", "ms_per_step": ms,
                                        "kernels_per_step": kps,
                                        "newton_iters_per_marker": sum(x["iterations"] for x in st) / max(mk, 1),
                                        "fallbacks_per_step": sum(x["fallbacks"] for x in st),
                                        "max_residual": max(x["max_residual"] for x in st),
                                        "tc_timeouts": sum(x["tc_timeouts"] for x in st)}
    for sched in ("per_member", "batched", "batched_1group"):
        out["speedup_surrogate_vs_plain_" + sched] = (out["surrogate_tc_" + sched]["value"] /
                                                      out["plain_" + sched]["value"])
    for label in ("plain", "surrogate_tc"):
        for sched in ("batched", "batched_1group"):
            out["speedup_%s_vs_per_member_%s" % (sched, label)] = (out[label + "_" + sched]["value"] /
                                                                   out[label + "_per_member"]["value"])
    E.close()
    for P in members:
        P.close()
    return out


def systems_leg(args, local):
    """The solves between the marker passes, on the device: the Stokes (formVEPSystem) and thermal
    (formThermalSystem) assembly and the direct solve (banded LU; the reference runs MUMPS LU) of
    the subduction box at 129 x 33 and 513 x 129 nodes, beside a host sparse LU (SuperLU) of the
    same matrices; then whole time steps (mic_subduction_timestep) of the 129 x 33 box with 16
    markers per cell."""
    import numpy as np
    import torch

    from fvmic2d_gb300 import gpu
    from fvmic2d_gb300 import workloads as W

    out = {"workload": "subduction_box: refined VEP box, slab at 0.8 rad below a 0.3 LY plate, 5 cm/yr inflow"}
    try:
        import scipy.sparse as sps
        import scipy.sparse.linalg as spl
    except ImportError:
        sps = None
    for ncx, ncy in ((128, 32), (512, 128)):
        wl, topt = W.subduction_box(nx_cells=ncx, ny_cells=ncy, nm=2)
        G = gpu.MicProblem(wl, device=local)
        G.findMarkerCells()
        G.updateMarkerRho()
        G.projectMarkersNodesAll2()
        st = torch.cuda.ExternalStream(G.stream(), device=local)
        rec = {"nodes": [wl.grid.NX, wl.grid.NY]}
        for which, name in ((G.STOKES, "stokes"), (G.THERMAL, "thermal")):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            if which == G.STOKES:
                G.formVEPSystem(topt.sub, topt.dtMax)
                G.linear_solve(which)  # warm-up
                G.synchronize()
                ev[0].record(st)
                G.formVEPSystem(topt.sub, topt.dtMax)
            else:
                G.enforceThermalBCs1(topt.sub)
                G.formThermalSystem(topt.sub, topt.dtMax)
                G.linear_solve(which)
                G.synchronize()
                ev[0].record(st)
                G.formThermalSystem(topt.sub, topt.dtMax)
            ev[1].record(st)
            G.linear_solve(which)
            ev[2].record(st)
            ev[2].synchronize()
            kl, ku = G.system_band(which)
            rp, c, v, rhs = G.system(which)
            r = {"unknowns": int(len(rhs)), "band": [kl, ku], "assembly_ms": ev[0].elapsed_time(ev[1]),
                 "solve_ms": ev[1].elapsed_time(ev[2])}
            if sps is not None:
                A = sps.csr_matrix((v, c, rp), shape=(len(rhs), len(rhs))).tocsc()
                t0 = time.perf_counter()
                xr = spl.spsolve(A, rhs)
                r["host_superlu_ms"] = (time.perf_counter() - t0) * 1e3
                x = G.solution(which)
                r["rel_diff_vs_superlu"] = float(np.max(np.abs(x - xr)) / np.max(np.abs(xr)))
            rec[name] = r
        G.close()
        out["%dx%d" % (wl.grid.NX, wl.grid.NY)] = rec
    wl, topt = W.subduction_box(nx_cells=128, ny_cells=32, nm=4)
    G = gpu.MicProblem(wl, device=local)
    G.subductionTimestep(topt, 0.0)  # warm-up step
    topt.firstStep = 0
    steps = 3
    t0 = time.perf_counter()
    reps = [G.subductionTimestep(topt, 0.0) for _ in range(steps)]
    ms = (time.perf_counter() - t0) * 1e3 / steps
    out["timestep"] = {"nodes": [wl.grid.NX, wl.grid.NY], "markers": int(G.n), "steps": steps,
                       "ms_per_step": ms, "plastic_iterations": [r["plastic_iterations"] for r in reps],
                       "dt": [r["dt"] for r in reps],
                       "note": "host wall time of mic_subduction_timestep: density control off, every "
                               "plasticity iteration assembles and solves the Stokes system on the device"}
    G.close()
    # Monte-Carlo members (fvmic2d's iMonte loop runs them one after another): 16 independent
    # 129 x 33 boxes with different slab angles, one step each, one member at a time and all of
    # them from host threads side by side (mic_subduction_timestep_many)
    members = []
    for k in range(16):
        wl, topt = W.subduction_box(nx_cells=128, ny_cells=32, nm=4, seed=10 + k)
        topt.sub.slabAngle = 0.6 + 0.02 * k
        members.append((gpu.MicProblem(wl, device=local), topt))
    probs = [P for P, _ in members]
    topts = [t for _, t in members]
    gpu.subduction_timestep_many(probs, topts)  # warm-up step: buffers, captured factorisations
    for t in topts:
        t.firstStep = 0
    t0 = time.perf_counter()
    for P, t in members:
        P.subductionTimestep(t, 0.0)
    seq_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    gpu.subduction_timestep_many(probs, topts)
    par_ms = (time.perf_counter() - t0) * 1e3
    out["monte_carlo"] = {"members": len(members), "markers": int(sum(P.n for P in probs)),
                          "one_at_a_time_ms_per_step": seq_ms, "side_by_side_ms_per_step": par_ms,
                          "speedup": seq_ms / par_ms,
                          "note": "host wall time of one step of every member"}
    for P in probs:
        P.close()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
