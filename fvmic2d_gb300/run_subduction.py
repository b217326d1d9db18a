"""fvmic2d's subduction program (main_subduction.c) on one GPU, without PETSc or MPI.

The set-up and the time loop are the reference's, call for call, each on the device:

  set-up   resetNodalFields, resetMarkers, distributeMarkersUniformInDomain,
           initialConditionsVanKeken (which also sets the slab-velocity boundary conditions),
           findMarkerCells, projectMarkersNodesAll2 twice, enforceThermalBCs1,
           projectNodalFieldToMarkersS(lastT -> T), findMarkerCells   (main_subduction.c:176-202)
  loop     mic_subduction_timestep: density control, plasticity iterations around the Stokes
           solve, stress updates, thermal solve, sub-grid temperature, diagnostics, advection
           (main_subduction.c:227-460); markers saved in the reference's binary format every
           `save_every` steps (saveMarkersBinary, io.c:299)

Usage:  python -m fvmic2d_gb300.run_subduction --nx-cells 128 --ny-cells 32 --steps 10

The grid is the refined box of `workloads.vep_slab_box` and the geometry that of
`workloads.subduction_box`; materials come from the same workload (the initial conditions set
every marker to material 0, as the reference's do).
"""
import argparse
import json
import os
import time

from . import gpu
from . import workloads as W


def setup(P, sub, NMX, NMY, seed=0):
    """main_subduction.c:176-202 on the device; returns the marker count"""
    P.resetNodalFields()
    P.resetMarkers()
    n = P.distributeMarkersUniformInDomain(NMX, NMY, seed)
    P.initialConditionsVanKeken(sub)
    P.findMarkerCells()
    P.projectMarkersNodesAll2()
    P.projectMarkersNodesAll2()
    P.enforceThermalBCs1(sub)
    P.projectNodalFieldToMarkersS("lastT", "T")
    P.findMarkerCells()
    return n


def run(P, topt, steps, elapsed=0.0, save_every=0, out_dir=None, on_step=None):
    """the time loop (main_subduction.c:227-460): returns (elapsed time, reports)"""
    reports = []
    for it in range(steps):
        topt.firstStep = 1 if it == 0 else 0
        rep = P.subductionTimestep(topt, elapsed)
        reports.append(rep)
        if rep["stopped"]:
            break
        elapsed += rep["dt"]
        if on_step:
            on_step(it, rep, elapsed)
        if save_every and out_dir and (it % save_every == 0 or it == steps - 1):
            P.saveMarkersBinary(os.path.join(out_dir, "Markers.0.%d" % it), elapsed)
    return elapsed, reports


def make_problem(nx_cells, ny_cells, NMX, NMY, seed=0, max_mark_factor=1.5, density_control=True):
    """a context sized for the run (capacity maxMarkFactor x the initial markers, as
    main_subduction.c:123 sizes allocateMarkers) and the step options"""
    wl, topt = W.subduction_box(nx_cells=nx_cells, ny_cells=ny_cells, nm=min(NMX, NMY), seed=seed)
    topt.densityControl = 1 if density_control else 0
    topt.density.NMX, topt.density.NMY = NMX, NMY
    so = topt.sub
    for f in ("slabAngle", "slabAge", "overridingPlateThickness", "rootThickness", "rootCenter", "rootWidth"):
        setattr(topt.density, f, getattr(so, f))
    cap = int(max_mark_factor * NMX * NMY * nx_cells * ny_cells) + 64
    return gpu.MicProblem(wl, capacity=cap), topt


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--nx-cells", type=int, default=128)
    ap.add_argument("--ny-cells", type=int, default=32)
    ap.add_argument("--nmx", type=int, default=4, help="markers per cell along x at set-up")
    ap.add_argument("--nmy", type=int, default=4)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--save-every", type=int, default=0, help="save markers every this many steps (0: never)")
    ap.add_argument("--out", default="output", help="directory for the marker files")
    ap.add_argument("--no-density-control", action="store_true")
    args = ap.parse_args()
    P, topt = make_problem(args.nx_cells, args.ny_cells, args.nmx, args.nmy,
                           density_control=not args.no_density_control)
    if args.save_every:
        os.makedirs(args.out, exist_ok=True)
    n = setup(P, topt.sub, args.nmx, args.nmy)
    t0 = time.perf_counter()

    def show(it, rep, elapsed):
        print(json.dumps({"step": it, "dt": rep["dt"], "elapsed": elapsed, "plastic_iterations":
                          rep["plastic_iterations"], "residual": rep["residual"], "nusselt": rep["nusselt"],
                          "vrms": rep["vrms"], "markers_added": rep["markers_added"], "max_T": rep["max_T"]}),
              flush=True)

    elapsed, reps = run(P, topt, args.steps, save_every=args.save_every, out_dir=args.out, on_step=show)
    print(json.dumps({"markers_at_setup": n, "steps": len(reps), "elapsed_time": elapsed,
                      "wall_seconds": time.perf_counter() - t0}), flush=True)
    P.close()


if __name__ == "__main__":
    main()
