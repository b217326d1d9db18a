"""Generate the golden vectors in this directory from fvmic2d's OWN hot-path C.

The reference sources are compiled against the single-rank petsc_lite stand-in by
oracle/build_ref.sh (needs the reference tree, so this runs only where it exists).
Each fixture records seeded inputs and the reference's outputs after every entry
point of one marker-path step, so the CPU oracle and the GPU kernels can be
checked against the reference anywhere, including machines without the tree.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fvmic2d_gb300 import workloads as W  # noqa: E402
from fvmic2d_gb300.mic_types import PROJECTED_FIELDS  # noqa: E402
from oracle import build as obuild  # noqa: E402
from oracle import refpy  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def edge_case_workload():
    """Small VEP box whose markers include the reference's corner cases: markers exactly on
    gridlines and cell centres (0.5 ties), at X = LX and Y = LY (cell NX-2 / NY-2,
    markers.c:49-59), outside the domain and NaN (cellX = -1), and one material per
    viscosity law and plasticity mode."""
    wl = W.vep_slab_box(nx_cells=12, ny_cells=6, nm=2, seed=7)
    g = wl.grid
    m = wl.markers
    extra = np.zeros(24, dtype=m.dtype)
    pts = [
        (g.x[3], g.y[2]), (g.x[5], g.yc[3]), (g.xc[4], g.y[4]), (g.xc[6], g.yc[2]),  # gridlines / centres
        (g.LX, g.y[3]), (g.x[2], g.LY), (g.LX, g.LY), (0.0, 0.0), (-0.0, g.yc[1]),
        (0.5 * (g.x[7] + g.x[8]), 0.5 * (g.y[1] + g.y[2])),  # exact 0.5 offsets
        (-1.0, g.yc[2]), (g.LX * 1.0000001, g.yc[2]), (g.xc[3], -5.0), (np.nan, g.yc[2]),
    ]
    for k, (x, y) in enumerate(pts):
        extra[k]["X"], extra[k]["Y"] = x, y
    rng_u = W.splitmix64_uniform(99, 2 * 24)
    for k in range(len(pts), len(extra)):
        extra[k]["X"] = rng_u[2 * k] * g.LX
        extra[k]["Y"] = rng_u[2 * k + 1] * g.LY
    for f in ("T", "eta", "mu", "sxx", "syy", "sxy", "exx", "eyy", "exy", "p", "Eii"):
        extra[f] = np.resize(m[f], len(extra))
    extra["Mat"] = np.arange(len(extra)) % 6
    m = np.concatenate([m, extra])
    m["Mat"][: len(m) - len(extra)] = np.arange(len(m) - len(extra)) % 6
    m["Eii"] = np.linspace(0.0, 2.0, len(m))
    mat = wl.materials
    mat.nMaterials = 6
    laws = [0, 1, 2, 3, 5, 6]
    for k in range(6):
        mat.materialEta[k] = [1e21, 1e21, 1e22, 1e18, 1e22, 1e21][k]
        mat.materialRho[k] = 3300.0 + 10 * k
        mat.materialkThermal[k] = 3.0 + 0.1 * k
        mat.materialCp[k] = 1250.0 - 5 * k
        mat.materialAlpha[k] = 3e-5
        mat.materialMu[k] = 1e10
        mat.hasEtaT[k] = laws[k]
        mat.QonR[k] = 2.0e4 if k != 4 else 1e-3
        mat.Tref[k] = 1573.0
    mat.hasPlasticity[1] = 1
    mat.materialCohesion[1] = 1e7
    mat.materialFriction[1] = 0.6
    mat.hasPlasticity[2] = 2  # strain weakening between gamma0 and gamma1
    mat.gamma[2][0], mat.gamma[2][1] = 0.5, 1.5
    mat.C[2][0], mat.C[2][1] = 2e7, 1e6
    mat.F[2][0], mat.F[2][1] = 30.0, 10.0
    mat.hasPlasticity[3] = 3  # unknown mode: yield stress 0
    opt = wl.options
    opt.slabAngle = 0.7
    opt.decoupleThickness = 3e4
    opt.minDecoupleDepth = 1e4
    opt.maxDecoupleDepth = 6e4
    opt.decoupleEtaScaler = 0.1
    wl.markers = m
    # prescribed-velocity walls exercise the ghost-velocity branches of advectMarkersRK
    wl.bcs.mechBCTop.type[0] = 0
    wl.bcs.mechBCTop.value[0] = 1e-10
    wl.bcs.mechBCLeft.type[1] = 0
    wl.bcs.mechBCLeft.value[1] = -2e-10
    wl.name = "edge_cases"
    return wl


def record(wl, steps=2, jaumann=False):
    """Run `steps` reference steps; store inputs and the state after every entry point.
    jaumann: the reference built with -DJAUMANN (advectMarkersRK's first-order stress rotation)."""
    p = refpy.RefProblem(wl, jaumann=jaumann)
    out = {"x": wl.grid.x, "y": wl.grid.y, "LX": wl.grid.LX, "LY": wl.grid.LY,
           "markers_in": wl.markers.copy(), "dt": wl.dt, "dt_thermal": wl.dt_thermal,
           "jaumann": np.int32(1 if jaumann else 0)}
    for name, arr in wl.nodal.items():
        out["nodal_in_" + name] = np.asarray(arr, dtype=np.float64)
    D = wl.options.subgridStressDiffusivity
    for s in range(steps):
        pre = "s%d_" % s
        out[pre + "nout"] = p.findMarkerCells()
        out[pre + "after_find"] = p.markers.copy()
        p.updateMarkerRho()
        p.projectMarkersNodesAll2()
        for f in PROJECTED_FIELDS:
            out[pre + "proj1_" + f] = p.get_nodal(f)
        out[pre + "maxT"] = p.maxMarkerT()
        out[pre + "yield"] = p.checkPlasticYielding(wl.dt)
        out[pre + "after_yield"] = p.markers.copy()
        p.limitViscosity()
        p.projectMarkersNodesAll2()
        for f in PROJECTED_FIELDS:
            out[pre + "proj2_" + f] = p.get_nodal(f)
        p.updateMarkerStrainPressure(wl.dt)
        out[pre + "after_strain"] = p.markers.copy()
        out[pre + "residual"] = p.updateGlobalStrainRateResidual(0)
        if D > 0:
            p.subgridStressChanges(wl.dt, D)
            out[pre + "after_subgrid_stress"] = p.markers.copy()
            for f in ("dsxx", "dsyy", "dsxy"):
                out[pre + "ds_" + f] = p.get_nodal(f)
        p.updateMarkerStress()
        out[pre + "after_stress"] = p.markers.copy()
        p.subgridTemperatureChanges(wl.dt_thermal)
        out[pre + "after_subgrid_T"] = p.markers.copy()
        p.advectMarkersRK(wl.dt_thermal)
        out[pre + "after_advect"] = p.markers.copy()
        out[pre + "maxSxx"] = p.maxAbsSxx()
    p.close()
    return out


def tables(wl):
    m, o, b = wl.materials, wl.options, wl.bcs
    return {"materials_bytes": np.frombuffer(bytes(m), dtype=np.uint8),
            "options_bytes": np.frombuffer(bytes(o), dtype=np.uint8),
            "bcs_bytes": np.frombuffer(bytes(b), dtype=np.uint8)}


def creep_table():
    """viscosity.c:106-179 on a grid over the composite-creep workload ranges, including the
    T = 255 K and 258 K parameter switches and the s < 1 Pa early return."""
    s = np.concatenate([[0.0, 0.5, 0.999999, 1.0, 1.000001], np.logspace(0, 8, 23)])
    T = np.array([100.0, 180.0, 254.999, 255.0, 257.0, 258.0, 265.0, 273.0])
    d = np.array([1e-4, 1e-3, 1e-2, 1e-1])
    P = np.array([0.0, 0.5, 1.0, 1e6, 1e8])
    S, TT, DD, PP = np.meshgrid(s, T, d, P, indexing="ij")
    eta = refpy.goldsby_kohlstedt(S.ravel(), TT.ravel(), DD.ravel(), PP.ravel())
    return {"s": S.ravel(), "T": TT.ravel(), "d": DD.ravel(), "P": PP.ravel(), "eta": eta}


def lifecycle_table():
    """resetMarkers + distributeMarkersUniformInDomain (markers.c:332-400) on a uniform and a
    refined grid at two marker densities: the reference's marker arrays (capacity included)."""
    out = {}
    for tag, wl in (("uniform", W.convection_box(ncell=8, nm=4, seed=1)),
                    ("refined", W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=2))):
        R = refpy.RefProblem(wl)
        for NMX, NMY in ((4, 4), (3, 5)):
            mk, n = R.distribute_uniform(NMX, NMY)
            key = "%s_%dx%d" % (tag, NMX, NMY)
            out[key + "_markers"] = _fields_only(mk).view(np.uint8).reshape(len(mk), -1)
            out[key + "_n"] = np.int64(n)
        out[tag + "_x"], out[tag + "_y"] = wl.grid.x, wl.grid.y
        out[tag + "_L"] = np.array([wl.grid.LX, wl.grid.LY])
    return out


def _fields_only(a):
    """the same markers with padding bytes zeroed (numpy leaves them arbitrary on copies)"""
    out = np.zeros(len(a), dtype=a.dtype)
    for f in a.dtype.names:
        out[f] = a[f]
    return out


def density_table():
    """checkMarkerDensity (markers.c:455-781) on the density case at two seeds: markers before
    (cells current) and after, capacity, and the drand48 state after.  The reference leaves cpu
    and strainRateResidual of the inflow markers it creates uninitialised; they are zeroed here."""
    out = {}
    for seed in (1, 77):
        wl, dopt = W.density_case()
        R = refpy.RefProblem(wl)
        R.findMarkerCells()
        before = R.markers.copy()
        cap = len(before) + 400
        after, state = R.checkMarkerDensity(dopt, cap, seed=seed)
        new = np.ones(len(after), dtype=bool)
        new[:len(before)] = ~np.all(after[:len(before)].view(np.uint8).reshape(len(before), -1) ==
                                    before.view(np.uint8).reshape(len(before), -1), axis=1)
        g, d = wl.grid, dopt
        plate = d.overridingPlateThickness + (d.rootThickness * np.cos(np.pi * (g.LX - d.rootCenter) / d.rootWidth / 2) ** 2
                                              if abs(g.LX - d.rootCenter) < d.rootWidth else 0.0)
        special = new & ((after["X"] < g.x[1]) | ((after["X"] >= g.x[-2]) & (after["Y"] >= plate)))
        after = after.copy()
        after["cpu"][special] = 0
        after["srr"][special] = 0.0
        key = "seed%d" % seed
        before, after = _fields_only(before), _fields_only(after)
        out[key + "_before"] = before.view(np.uint8).reshape(len(before), -1)
        out[key + "_after"] = after.view(np.uint8).reshape(len(after), -1)
        out[key + "_special"] = special
        out[key + "_cap"] = np.int64(cap)
        out[key + "_state"] = np.uint64(state)
    out["options_bytes"] = np.frombuffer(bytes(dopt), dtype=np.uint8)
    return out


def grid_table():
    """nodalStressStrain, limitDisplacementTimestep and retrieveSolutions of the reference on
    the grid cases of tests/test_oracle_pin.py (inputs and outputs)."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.test_oracle_pin import GRID_OUT, grid_case

    out = {}
    for kind, seed in (("free_slip", 5), ("prescribed", 8)):
        wl, S = grid_case(kind, seed)
        R = refpy.RefProblem(wl)
        for name, arr in wl.nodal.items():
            out["%s_in_%s" % (kind, name)] = np.asarray(arr, dtype=np.float64)
        out[kind + "_bcs"] = np.frombuffer(bytes(wl.bcs), dtype=np.uint8)
        R.nodalStressStrain(3.0e11)
        for name in GRID_OUT:
            out["%s_out_%s" % (kind, name)] = R.get_nodal(name)
        out[kind + "_dt"] = np.array([R.limitDisplacementTimestep(1e14, 0.5), R.limitDisplacementTimestep(1e30, 0.1)])
        out[kind + "_S"] = S
        R.retrieveSolutions(S, 1e20)
        for name in ("vx", "vy", "p"):
            out["%s_ret_%s" % (kind, name)] = R.get_nodal(name)
    return out


def systems_table():
    """formVEPSystem, enforceThermalBCs1 and formThermalSystem of the reference on the systems
    cases of tests/test_oracle_pin.py: inputs, the matrices as CSR, right-hand sides, Kbond and
    Kcont, and lastT after the boundary values."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.test_oracle_pin import SYSTEM_IN, SYSTEM_KINDS, reference_systems, systems_case

    out = {}
    for kind in SYSTEM_KINDS:
        wl, so, dt = systems_case(kind)
        for name in SYSTEM_IN:
            out["%s_in_%s" % (kind, name)] = np.asarray(wl.nodal[name], dtype=np.float64)
        (rp, c, v, rhs, kb, kc), lastT, (trp, tc, tv, trhs) = reference_systems(wl, so, dt)
        for name, a in (("rowptr", rp), ("cols", c), ("vals", v), ("rhs", rhs)):
            out["%s_stokes_%s" % (kind, name)] = a
        out[kind + "_K"] = np.array([kb, kc])
        out[kind + "_lastT"] = lastT
        for name, a in (("rowptr", trp), ("cols", tc), ("vals", tv), ("rhs", trhs)):
            out["%s_thermal_%s" % (kind, name)] = a
    return out


def timestep_table():
    """one time step of main_subduction.c through the reference's routines (host LU solves):
    markers before and after, the step's scalars and the final nodal velocity, pressure and
    temperature"""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.timestep_case import reference_timestep, timestep_case

    from tests.timestep_case import timestep_density_case

    out = {}
    wl, topt = timestep_case()
    cases = [("", wl, topt, None)]
    wl2, topt2, cap2 = timestep_density_case()
    cases.append(("dens_", wl2, topt2, cap2))
    from tests.timestep_case import timestep_adiabatic_case

    wl3, topt3 = timestep_adiabatic_case()
    cases.append(("adiab_", wl3, topt3, None))
    for pre, w, t, cap in cases:
        before = np.array(w.markers, copy=True)
        mk, rep, nodal = reference_timestep(w, t, elapsed=0.0, capacity=cap)
        out[pre + "before"] = before.view(np.uint8)
        out[pre + "after"] = mk.view(np.uint8)
        for k, v in rep.items():
            out[pre + "rep_" + k] = np.array(v)
        for k, v in nodal.items():
            out[pre + "nodal_" + k] = v
    return out


def run_table():
    """main_subduction.c's set-up and first two time steps through the reference's routines (host
    LU solves) on the small subduction box: markers after set-up and after each step, the step
    reports"""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.timestep_case import reference_run, run_case

    wl, topt, nmx, nmy, steps = run_case()
    setup, mks, reps = reference_run(wl, topt, nmx, nmy, steps)
    out = {"setup": setup.view(np.uint8)}
    for i, (mk, rep) in enumerate(zip(mks, reps)):
        out["step%d" % i] = mk.view(np.uint8)
        for k, v in rep.items():
            out["rep%d_%s" % (i, k)] = np.array(v)
    return out


def adiabatic_table():
    """adiabaticHeating of the reference plus main's addition to the heating field"""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.test_oracle_pin import adiabatic_case

    wl, gy = adiabatic_case()
    R = refpy.RefProblem(wl)
    R.findMarkerCells()
    R.adiabaticHeating(gy)
    return {"before": np.array(wl.markers, copy=True).view(np.uint8), "heat_in": wl.nodal["heating"],
            "heat_out": R.get_nodal("heating")}


def diagnostics_table():
    """nusseltNumber and rmsVelocity (post.c) of the reference on the diagnostics case"""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.test_oracle_pin import diagnostics_case

    wl, bottom, top = diagnostics_case()
    R = refpy.RefProblem(wl)
    out = {"in_" + f: np.asarray(wl.nodal[f], dtype=np.float64) for f in ("thisT", "vx", "vy")}
    out["nusselt"] = np.array(R.nusseltNumber(bottom, top))
    out["vrms"] = np.array(R.rmsVelocity())
    return out


def van_keken_table():
    """initialConditionsVanKeken of the reference: markers before and after, the BCs it sets"""
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tests.test_oracle_pin import van_keken_case

    wl, so = van_keken_case()
    before = np.array(wl.markers, copy=True)
    R = refpy.RefProblem(wl)
    b = R.initialConditionsVanKeken(so)
    return {"before": before.view(np.uint8), "after": R.markers.view(np.uint8),
            "bcs": np.frombuffer(bytes(b), dtype=np.uint8)}


def checkpoint_case():
    """the VEP box after a step, with some markers pushed out of the domain"""
    wl = W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=2)
    m = wl.markers
    m["X"][::37] = -1.0
    m["Y"][5::41] = wl.grid.LY * 1.5
    return wl


def checkpoint_table():
    """saveMarkersBinary / restartFromMarkers (io.c:299, restart.c:8) of the reference: input
    markers (cells found), the file's bytes, and the markers restarted from it."""
    import tempfile

    wl = checkpoint_case()
    R = refpy.RefProblem(wl)
    R.findMarkerCells()
    before = _fields_only(R.markers)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        try:
            os.mkdir("output")
            R.saveMarkersBinary(0, 7, 1.25e13)
            raw = np.fromfile(os.path.join("output", "Markers.0.7"), dtype=np.uint8)
            t = R.restartFromMarkers(0, 7, len(before) + 10)
        finally:
            os.chdir(cwd)
    after = _fields_only(R.markers)
    after["srr"] = 0.0  # never read from the file; the reference leaves it as allocated
    return {"markers_in": before.view(np.uint8).reshape(len(before), -1), "file_bytes": raw,
            "restart": after.view(np.uint8).reshape(len(after), -1), "elapsed": np.float64(t)}


def main():
    if obuild.build_ref() is None:
        raise SystemExit("reference tree not found; golden vectors can only be generated where it exists")
    if sys.argv[1:] in ([], ["lifecycle"]):
        np.savez_compressed(os.path.join(OUT, "marker_lifecycle.npz"), **lifecycle_table())
        print("wrote marker_lifecycle")
    if sys.argv[1:] in ([], ["density"]):
        np.savez_compressed(os.path.join(OUT, "marker_density.npz"), **density_table())
        print("wrote marker_density")
    if sys.argv[1:] in ([], ["checkpoint"]):
        np.savez_compressed(os.path.join(OUT, "marker_checkpoint.npz"), **checkpoint_table())
        print("wrote marker_checkpoint")
    if sys.argv[1:] in ([], ["timestep"]):
        np.savez_compressed(os.path.join(OUT, "subduction_step.npz"), **timestep_table())
        print("wrote subduction_step")
    if sys.argv[1:] in ([], ["run"]):
        np.savez_compressed(os.path.join(OUT, "subduction_run.npz"), **run_table())
        print("wrote subduction_run")
    if sys.argv[1:] in ([], ["vankeken"]):
        np.savez_compressed(os.path.join(OUT, "van_keken.npz"), **van_keken_table())
        print("wrote van_keken")
    if sys.argv[1:] in ([], ["diagnostics"]):
        np.savez_compressed(os.path.join(OUT, "post_diagnostics.npz"), **diagnostics_table())
        print("wrote post_diagnostics")
    if sys.argv[1:] in ([], ["adiabatic"]):
        np.savez_compressed(os.path.join(OUT, "adiabatic_heating.npz"), **adiabatic_table())
        print("wrote adiabatic_heating")
    if sys.argv[1:] in ([], ["systems"]):
        np.savez_compressed(os.path.join(OUT, "linear_systems.npz"), **systems_table())
        print("wrote linear_systems")
    if sys.argv[1:] in ([], ["grid"]):
        np.savez_compressed(os.path.join(OUT, "grid_routines.npz"), **grid_table())
        print("wrote grid_routines")
    if sys.argv[1:] in ([], ["periodic"]):
        # the marker path on a grid periodic in x (gridGenerator.c:67-68), markers crossing the seam
        wl = W.periodic_box(nx_cells=16, ny_cells=6, nm=3, seed=9)
        rec = record(wl, steps=3)
        rec.update(tables(wl))
        np.savez_compressed(os.path.join(OUT, "periodic_box.npz"), **rec)
        print("wrote periodic_box", len(wl.markers), "markers")
    if sys.argv[1:] in ([], ["jaumann"]):
        # the same path with the reference's compile-time JAUMANN stress rotation (markers.c:2147-2156)
        wl = W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=12)
        rec = record(wl, steps=2, jaumann=True)
        rec.update(tables(wl))
        np.savez_compressed(os.path.join(OUT, "vep_jaumann.npz"), **rec)
        print("wrote vep_jaumann", len(wl.markers), "markers")
    if sys.argv[1:]:
        return
    cases = {
        "convection_box_8": W.convection_box(ncell=8, nm=4, seed=1),
        "vep_slab_box_16x4": W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=2),
        "edge_cases": edge_case_workload(),
    }
    for name, wl in cases.items():
        rec = record(wl, steps=2)
        rec.update(tables(wl))
        np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
        print("wrote", name, len(wl.markers), "markers")
    np.savez_compressed(os.path.join(OUT, "goldsby_kohlstedt.npz"), **creep_table())
    print("wrote goldsby_kohlstedt")


if __name__ == "__main__":
    main()
