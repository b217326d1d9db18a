"""One time step of main_subduction.c (227-460) as a case: the workload, the step options, and
the reference's own routines called in main's order with host sparse LU solves standing in for
MUMPS (test infrastructure: generates and checks tests/golden/subduction_step.npz)."""
import contextlib
import os

import numpy as np

from fvmic2d_gb300 import workloads as W
from fvmic2d_gb300.mic_types import NF, DensityOptions, TimestepOptions
from tests.test_oracle_pin import systems_case


def timestep_case(seed=4):
    """the refined VEP box with 4 x 4 markers per cell, subduction boundary geometry (slab at
    0.8 rad below a plate 0.3 LY thick) and the step settings"""
    wl = W.vep_slab_box(nx_cells=24, ny_cells=10, nm=4, seed=seed)
    _, so, _ = systems_case("fixed_top")
    g = wl.grid
    so.overridingPlateThickness = 0.3 * g.LY
    so.rootCenter = 0.5 * g.LX
    so.rootWidth = 0.2 * g.LX
    so.rootThickness = 0.05 * g.LY
    topt = TimestepOptions(dtMax=3.0e11, displacementStepLimit=0.5, maxTempChange=50.0, maxNumPlasticity=4,
                           shearHeating=1, firstStep=1, densityControl=0,
                           density=DensityOptions(NMX=4, NMY=4, minMarkers=1, maxMarkers=100), sub=so,
                           thermalBCBottomValue=1573.0)
    return wl, topt


def timestep_density_case(seed=6):
    """the same box with density control in the step (main_subduction.c:250): markers emptied
    from a block of cells inside the wedge and from the first cell column (the reference then adds
    subduction-inflow markers there), drand48 stream at srand48(1), main's seed"""
    wl, topt = timestep_case(seed=seed)
    g, m = wl.grid, wl.markers
    gone = ((m["X"] > g.x[12]) & (m["X"] < g.x[15]) & (m["Y"] > g.y[5]) & (m["Y"] < g.y[7])) | (m["X"] < g.x[1])
    m["X"][gone] = -1.0
    m["Y"][gone] = -1.0
    so = topt.sub
    topt.densityControl = 1
    topt.density = DensityOptions(NMX=4, NMY=4, minMarkers=1, maxMarkers=100, slabAngle=so.slabAngle,
                                  slabAge=so.slabAge, overridingPlateThickness=so.overridingPlateThickness,
                                  rootThickness=so.rootThickness, rootCenter=so.rootCenter, rootWidth=so.rootWidth)
    return wl, topt, len(m) + 4096


def timestep_adiabatic_case(seed=7):
    """the box with adiabatic heating on (main_subduction.c:374-378) and the markers moving
    vertically, as a previous advection would have left them"""
    wl, topt = timestep_case(seed=seed)
    m = wl.markers
    m["VY"] = (W.splitmix64_uniform(seed + 50, len(m)) - 0.5) * 2e-9
    topt.adiabaticHeating = 1
    return wl, topt


def _spsolve(rp, c, v, rhs):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    n = len(rp) - 1
    return spl.spsolve(sp.csr_matrix((v, c, rp), shape=(n, n)).tocsc(), rhs)


def reference_timestep(wl, topt, elapsed=0.0, capacity=None):
    """main_subduction.c:241-438 with the reference build's routines; returns (markers after the
    step, report dict, nodal fields dict)"""
    from oracle import refpy

    R = refpy.RefProblem(wl)
    return reference_step(R, topt, elapsed, capacity)


def reference_step(R, topt, elapsed=0.0, capacity=None):
    """one pass of main's time loop on an existing reference problem"""
    from oracle import refpy

    so = topt.sub
    with open(os.devnull, "w") as devnull, contextlib.redirect_stdout(devnull):
        R.findMarkerCells()
        added = 0
        if topt.densityControl:
            n0 = len(R.markers)
            out0 = int(np.sum(R.markers["cellX"] == -1))
            R.checkMarkerDensity(topt.density, capacity, seed=1)
            R.findMarkerCells()
            added = len(R.markers) - n0 + out0 - int(np.sum(R.markers["cellX"] == -1))
        R.updateMarkerRho()
        R.projectMarkersNodesAll2()
        rep = {"max_T": R.maxMarkerT(), "markers_added": added}
        ddt = topt.dtMax
        is_y, conv, it = 1, 0, 0
        kb = kc = res = 0.0
        while (topt.firstStep and it < 1) or ((is_y or not conv) and it < topt.maxNumPlasticity):
            is_y = R.checkPlasticYielding(ddt, elapsed)
            R.limitViscosity()
            R.projectMarkersNodesAll2()
            rp, c, v, rhs, kb, kc = R.formVEPSystem(so, ddt)
            R.retrieveSolutions(_spsolve(rp, c, v, rhs), kc)
            R.nodalStressStrain(ddt, so.gy)
            R.updateMarkerStrainPressure(ddt)
            res = R.updateGlobalStrainRateResidual(it)
            conv = refpy.lib().ref_checkConvergence(1e-16, 1e-1, it)
            last = ddt
            ddt = R.limitDisplacementTimestep(ddt, topt.displacementStepLimit)
            if ddt != last:
                conv = 0
            it += 1
        rep.update(plastic_iterations=it, is_yielding=is_y, converged=conv, displacement_dt=ddt, Kbond=kb,
                   Kcont=kc, residual=res)
        dt = ddt
        if R.wl.options.subgridStressDiffusivity > 0.0:
            R.subgridStressChanges(ddt, R.wl.options.subgridStressDiffusivity)
        R.updateMarkerStress()
        if not topt.shearHeating:
            R.set_nodal("heating", np.zeros((R.NY, R.NX)))
        if topt.adiabaticHeating:
            R.adiabaticHeating(so.gy)

        def thermal(dt):
            R.enforceThermalBCs1(so)
            rp, c, v, rhs = R.formThermalSystem(so, dt)
            T = _spsolve(rp, c, v, rhs)
            R.set_nodal("thisT", T.reshape(R.NY, R.NX))
            return np.max(np.abs(T - R.get_nodal("lastT").ravel()))

        dTmax = thermal(dt)
        rep["thermal_resolves"] = 0
        if dTmax > topt.maxTempChange:
            dt = dt * topt.maxTempChange / dTmax
            dTmax = thermal(dt)
            rep["thermal_resolves"] = 1
        rep.update(dt=dt, max_temp_change=dTmax)
        R.subgridTemperatureChanges(dt)
        rep["nusselt"] = R.nusseltNumber(topt.thermalBCBottomValue, so.thermalBCTopValue)
        rep["vrms"] = R.rmsVelocity()
        R.advectMarkersRK(dt)
        rep["max_abs_sxx"] = R.maxAbsSxx()
        nodal = {f: R.get_nodal(f) for f in ("vx", "vy", "p", "thisT", "lastT", "etaS", "etaN", "heating")}
    return R.markers.copy(), rep, nodal


def reference_run(wl, topt, NMX, NMY, steps):
    """main_subduction.c from set-up (176-202) through `steps` passes of the time loop, with the
    reference build's routines and host sparse LU solves; density control off.  Returns the
    markers after set-up, the markers after every step and the step reports."""
    import ctypes

    from oracle import refpy

    so = topt.sub
    with open(os.devnull, "w") as devnull, contextlib.redirect_stdout(devnull):
        R = refpy.RefProblem(wl)
        for f in NF:  # resetNodalFields (nodalFields.c:155); the Vecs it leaves are zero from creation
            R.set_nodal(f, np.zeros((R.NY, R.NX)))
        mk, n = R.distribute_uniform(NMX, NMY)
        R.markers = mk[:n].copy()
        refpy.lib().ref_set_markers(R.h, R.markers.ctypes.data, len(R.markers))
        bcs = R.initialConditionsVanKeken(so)
        refpy.lib().ref_set_bcs(R.h, ctypes.byref(bcs))  # updateBoundaryConditions (updateBCs.c:9)
        R.findMarkerCells()
        R.projectMarkersNodesAll2()
        R.projectMarkersNodesAll2()
        R.enforceThermalBCs1(so)
        R.projectNodalFieldToMarkersS("lastT", "T")
        R.findMarkerCells()
    setup = R.markers.copy()
    out, reps, elapsed = [], [], 0.0
    for it in range(steps):
        topt.firstStep = 1 if it == 0 else 0
        mk, rep, _ = reference_step(R, topt, elapsed)
        elapsed += rep["dt"]
        out.append(mk)
        reps.append(rep)
    return setup, out, reps


def run_case():
    """the whole program on a small grid: the subduction box of 32 x 8 cells, 4 x 4 markers per
    cell at set-up, two steps, density control off"""
    wl, topt = W.subduction_box(nx_cells=32, ny_cells=8, nm=4, seed=4)
    topt.densityControl = 0
    return wl, topt, 4, 4, 2
