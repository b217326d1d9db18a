"""A whole time step of main_subduction.c on the device (mic_subduction_timestep: plasticity
iterations around the Stokes solve, stress and temperature updates, thermal solve with the step
cut when the temperature changes too much, advection) against the reference's own routines called
in main's order with a host sparse LU in MUMPS's place (golden vectors).  The two direct solves
round differently, so results agree to a tolerance instead of bit for bit."""
import os

import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from fvmic2d_gb300.mic_types import MARKER_DTYPE
from tests.timestep_case import timestep_adiabatic_case, timestep_case, timestep_density_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# relative to each field's largest magnitude: the solves agree to about 1e-12 relative, and the
# marker updates pass that on nearly unchanged
FIELD_RTOL = {"X": 1e-9, "Y": 1e-9, "T": 1e-9, "eta": 1e-7, "p": 1e-7, "s": 1e-7, "e": 1e-6, "Eii": 1e-7}


def _fields(m):
    return {"X": m["X"], "Y": m["Y"], "T": m["T"], "eta": m["eta"], "p": m["p"], "Eii": m["Eii"],
            "s": np.stack([m["sxx"], m["syy"], m["sxy"]], axis=-1),
            "e": np.stack([m["exx"], m["eyy"], m["exy"]], axis=-1)}


@pytest.mark.parametrize("build", ["exact", "product"])
@pytest.mark.parametrize("case", ["plain", "density", "adiabatic"])
def test_timestep_matches_reference(build, case):
    """plain: no density control; density: checkMarkerDensity inside the step fills an emptied
    block of the wedge and the first cell column (subduction-inflow markers) before the solves;
    adiabatic: adiabatic heating added to the shear heating before the thermal solve"""
    z = np.load(os.path.join(GOLDEN, "subduction_step.npz"))
    pre = {"plain": "", "density": "dens_", "adiabatic": "adiab_"}[case]
    cap = None
    if case == "plain":
        wl, topt = timestep_case()
    elif case == "density":
        wl, topt, cap = timestep_density_case()
    else:
        wl, topt = timestep_adiabatic_case()
    wl.markers = z[pre + "before"].view(MARKER_DTYPE).copy()
    ref = z[pre + "after"].view(MARKER_DTYPE)
    G = gpu.MicProblem(wl, exact=(build == "exact"), capacity=cap)
    rep = G.subductionTimestep(topt, 0.0)
    assert rep["stopped"] == 0
    assert rep["markers_added"] == int(z[pre + "rep_markers_added"])
    for k in ("plastic_iterations", "is_yielding", "converged", "thermal_resolves"):
        assert rep[k] == int(z[pre + "rep_" + k]), k
    for k in ("dt", "displacement_dt", "Kbond", "Kcont", "max_T", "max_temp_change", "max_abs_sxx", "nusselt",
              "vrms"):
        ref_v = float(z[pre + "rep_" + k])
        assert abs(rep[k] - ref_v) <= 1e-9 * abs(ref_v), (k, rep[k], ref_v)
    got = G.markers
    assert len(got) == len(ref)
    gf, rf = _fields(got), _fields(ref)
    worst = {}
    for k, tol in FIELD_RTOL.items():
        scale = np.max(np.abs(rf[k]))
        err = np.max(np.abs(gf[k] - rf[k])) / scale
        worst[k] = err
        assert err <= tol, (k, err, worst)
    for f in ("vx", "vy", "thisT"):
        a, b = G.get_nodal(f), z[pre + "nodal_" + f]
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b)), f


def test_timestep_stops_above_melting():
    """a marker above the reference's TBREAK (9999 K) ends the step after the projection, as main
    goes on to the next Monte-Carlo run: nothing is solved or advected"""
    wl, topt = timestep_case()
    wl.markers["T"][17] = 1.2e4
    G = gpu.MicProblem(wl)
    rep = G.subductionTimestep(topt, 0.0)
    assert rep["stopped"] == 1 and rep["max_T"] == 1.2e4
    assert rep["plastic_iterations"] == 0 and rep["dt"] == 0.0
    got = G.markers
    for f in ("X", "Y", "T", "sxx", "eta"):
        assert np.array_equal(got[f], wl.markers[f]), f


def _members(k_seeds=(4, 5, 6)):
    from fvmic2d_gb300 import workloads as W

    out = []
    for k, seed in enumerate(k_seeds):
        wl, topt = W.subduction_box(nx_cells=32, ny_cells=8, nm=4, seed=seed)
        topt.sub.slabAngle = 0.7 + 0.05 * k  # members differ in geometry as well as markers
        out.append((wl, topt))
    return out


def test_members_stepped_together_match_members_stepped_alone():
    """mic_subduction_timestep_many steps independent Monte-Carlo members from host threads side
    by side; each member's result is the one it gets stepped alone, bit for bit, over two steps"""
    alone, together = [], []
    for wl, topt in _members():
        alone.append((gpu.MicProblem(wl), topt))
        together.append(gpu.MicProblem(wl))
    rep_alone = []
    for step in range(2):
        for P, topt in alone:
            topt.firstStep = 1 if step == 0 else 0
            rep_alone.append(P.subductionTimestep(topt, 0.0))
    rep_many = []
    topts = [t for _, t in alone]
    for step in range(2):
        for t in topts:
            t.firstStep = 1 if step == 0 else 0
        rep_many += gpu.subduction_timestep_many(together, topts)
    assert rep_many == rep_alone
    for (P, _), Q in zip(alone, together):
        a, b = P.markers, Q.markers
        for f in ("X", "Y", "T", "sxx", "syy", "sxy", "eta", "p", "Eii"):
            assert np.array_equal(a[f], b[f]), f
        for f in ("vx", "vy", "p", "thisT"):
            assert np.array_equal(P.get_nodal(f), Q.get_nodal(f)), f


@pytest.mark.parametrize("build", ["exact", "product"])
def test_adiabatic_heating_matches_reference(build):
    """adiabaticHeating (adiabaticHeating.c:7) plus main's addition to the heating field: the
    projection sums in another order than the reference's marker loop (and multiplies the weight
    factors in another order), so the added heating agrees to 1e-12 of its largest value"""
    from tests.test_oracle_pin import adiabatic_case

    z = np.load(os.path.join(GOLDEN, "adiabatic_heating.npz"))
    wl, gy = adiabatic_case()
    wl.markers = z["before"].view(MARKER_DTYPE).copy()
    wl.nodal["heating"] = z["heat_in"]
    G = gpu.MicProblem(wl, exact=(build == "exact"))
    G.adiabaticHeating(gy)
    added, ref = G.get_nodal("heating") - z["heat_in"], z["heat_out"] - z["heat_in"]
    assert np.max(np.abs(added - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_static_velocity_reuses_the_first_solution():
    """Options.staticVelocity (main_subduction.c:306-318): the run's first step solves the Stokes
    system; later steps reuse that solution (same velocities, same Kcont) while the markers still
    go through their plasticity iterations and move"""
    wl, topt = timestep_case()
    topt.staticVelocity = 1
    G = gpu.MicProblem(wl)
    r1 = G.subductionTimestep(topt, 0.0)
    v1 = {f: G.get_nodal(f) for f in ("vx", "vy", "p")}
    x1 = G.markers["X"].copy()
    l0 = G.launch_count()
    topt.firstStep = 0
    r2 = G.subductionTimestep(topt, r1["dt"])
    for f in ("vx", "vy", "p"):
        assert np.array_equal(G.get_nodal(f), v1[f]), f
    assert (r2["Kbond"], r2["Kcont"]) == (r1["Kbond"], r1["Kcont"])
    assert r2["plastic_iterations"] >= 1
    assert not np.array_equal(G.markers["X"], x1)
    l_static = G.launch_count() - l0
    # the same two steps without staticVelocity: the second step solves again, with more launches
    wl2, topt2 = timestep_case()
    H = gpu.MicProblem(wl2)
    H.subductionTimestep(topt2, 0.0)
    topt2.firstStep = 0
    l1 = H.launch_count()
    H.subductionTimestep(topt2, r1["dt"])
    assert l_static < H.launch_count() - l1


def test_diagnostics_match_reference():
    """nusseltNumber (bit-identical: one thread sums in the reference's order) and rmsVelocity
    (a tree sum of the same terms: rounding only) against the reference's post.c"""
    from tests.test_oracle_pin import diagnostics_case

    z = np.load(os.path.join(GOLDEN, "post_diagnostics.npz"))
    wl, bottom, top = diagnostics_case()
    for f in ("thisT", "vx", "vy"):
        wl.nodal[f] = z["in_" + f]
    G = gpu.MicProblem(wl)
    assert G.nusseltNumber(bottom, top) == float(z["nusselt"])
    v = float(z["vrms"])
    assert abs(G.rmsVelocity() - v) <= 1e-14 * v


@pytest.mark.parametrize("build", ["exact", "product"])
def test_van_keken_initial_conditions_match_reference(build):
    """initialConditionsVanKeken (benchmarkInitialConditions.c:8): material, rhodot and the
    boundary conditions' types exact; temperature, density, viscosity and shear modulus within
    1e-12 (CUDA's erf, cos and exp against the host C library's)"""
    from fvmic2d_gb300.mic_types import BCs
    from tests.test_oracle_pin import van_keken_case

    z = np.load(os.path.join(GOLDEN, "van_keken.npz"))
    wl, so = van_keken_case()
    wl.markers = z["before"].view(MARKER_DTYPE).copy()
    ref = z["after"].view(MARKER_DTYPE)
    G = gpu.MicProblem(wl, exact=(build == "exact"))
    G.initialConditionsVanKeken(so)
    got = G.markers
    assert np.array_equal(got["Mat"], ref["Mat"]) and np.array_equal(got["rhodot"], ref["rhodot"])
    for f in ("T", "rho", "eta", "mu"):
        a, b = got[f], ref[f]
        assert np.all(np.abs(a - b) <= 1e-12 * np.abs(b)), f
    for f in ("X", "Y", "sxx", "p"):
        assert np.array_equal(got[f], ref[f]), f
    rb = BCs.from_buffer_copy(z["bcs"].tobytes())
    gb = G.get_bcs()
    for side in ("mechBCLeft", "mechBCTop"):  # the entries the routine sets: x and y of both
        g, r = getattr(gb, side), getattr(rb, side)
        assert list(g.type)[:2] == list(r.type)[:2], side
        assert np.allclose(list(g.value)[:2], list(r.value)[:2], rtol=1e-15, atol=0), side
