"""GPU parity: the CUDA marker path against the CPU oracle and the reference's golden vectors.

Three bars, all through the C ABI (libmic_gb300*.so):
* integer work (cell indices, out-of-domain counts, sort order, cell ranges): bit-exact;
* the FMA-free build (libmic_gb300_exact.so) against the oracle run on the markers in the
  GPU's sorted order: bit-exact wherever no CUDA transcendental is involved -- the sums
  are formed in the same order with the same roundings;
* the product build (libmic_gb300.so) against the reference order: relative 1e-12 with
  an absolute floor of 1e-12 x the field's largest magnitude (tests/helpers.py).
"""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from fvmic2d_gb300.mic_types import MARKER_DTYPE, PROJECTED_FIELDS
from oracle import oraclepy
from tests.helpers import compare_markers, exact, close, RTOL
from tests.test_oracle_pin import load_case, run_sequence, as_markers, is_jaumann

pytestmark = pytest.mark.gpu


def cell_keys(markers, NX, NY):
    k = markers["cellY"].astype(np.int64) * (NX - 1) + markers["cellX"]
    return np.where(markers["cellX"] < 0, (NX - 1) * (NY - 1), k)


def sort_keys(markers, grid):
    """The binning's sort key: 4 * cell + quadrant (qx = X >= xc[cellX+1], qy = Y >= yc[cellY+1]),
    out-of-domain markers last."""
    inside = markers["cellX"] >= 0
    cx = np.where(inside, markers["cellX"], 0).astype(np.int64)
    cy = np.where(inside, markers["cellY"], 0).astype(np.int64)
    with np.errstate(invalid="ignore"):
        qx = (markers["X"] >= grid.xc[cx + 1]).astype(np.int64)
        qy = (markers["Y"] >= grid.yc[cy + 1]).astype(np.int64)
    k = 4 * (cy * (grid.NX - 1) + cx) + 2 * qy + qx
    return np.where(inside, k, 4 * grid.ncells)


def transcendental_free(wl):
    """Same workload with every exp/sin/cos argument made exactly zero: constant viscosity
    laws, no subgrid diffusion, zero vorticity."""
    for k in range(wl.materials.nMaterials):
        wl.materials.hasEtaT[k] = 0
    wl.options.subgridStressDiffusivity = 0.0
    wl.options.subgridTemperatureDiffusivity = 0.0
    wl.nodal["wxy"] = np.zeros_like(wl.nodal["wxy"])
    return wl


class SortedOracle:
    """The oracle run on the markers in the GPU's current device order."""

    def __init__(self, wl):
        self.O = oraclepy.OracleProblem(wl)
        self.ids = np.arange(len(wl.markers), dtype=np.int64)

    def follow(self, ids):
        pos = np.empty_like(self.ids)
        pos[self.ids] = np.arange(len(self.ids))
        self.O.markers = self.O.markers[pos[ids]].copy()
        self.ids = ids.astype(np.int64)

    def caller_order(self):
        out = np.empty_like(self.O.markers)
        out[self.ids] = self.O.markers
        return out


# ---- binning and the stable counting sort -------------------------------------------


@pytest.mark.parametrize("name", ["convection_box_8", "vep_slab_box_16x4", "edge_cases"])
def test_find_cells_and_sort_match_stable_sort(name):
    wl, z = load_case(name)
    G = gpu.MicProblem(wl)
    nout = G.findMarkerCells()
    got = G.markers
    want = as_markers(z["s0_after_find"])
    assert nout == int(z["s0_nout"])
    for f in ("cellX", "cellY", "cpu"):
        ok, msg = exact(got[f], want[f])
        assert ok, f + " " + msg
    keys = cell_keys(want, wl.grid.NX, wl.grid.NY)
    ids = G.sorted_ids()
    np.testing.assert_array_equal(ids, np.argsort(sort_keys(want, wl.grid), kind="stable"))
    cs = G.cell_start()
    counts = np.bincount(keys, minlength=wl.grid.ncells + 1)
    np.testing.assert_array_equal(cs, np.concatenate([[0], np.cumsum(counts)]))
    assert G.status().n_out == nout


def test_second_binning_is_stable_in_device_order():
    wl = W.vep_slab_box(nx_cells=40, ny_cells=10, nm=4, seed=21)
    G = gpu.MicProblem(wl)
    G.findMarkerCells()
    ids0 = G.sorted_ids()
    G.advectMarkersRK(wl.dt_thermal * 3.0)
    G.findMarkerCells()
    ids1 = G.sorted_ids()
    mk = G.markers
    keys_prev_order = sort_keys(mk, wl.grid)[ids0]
    np.testing.assert_array_equal(ids1, ids0[np.argsort(keys_prev_order, kind="stable")])


def test_sort_many_cells_and_ragged_counts():
    """Random markers (empty and crowded cells, out-of-domain, NaN) on a grid with more
    cells than one radix digit covers: the permutation is a valid stable sort."""
    wl = W.convection_box(ncell=300, nm=1, seed=5)
    n = 200_000
    u = W.splitmix64_uniform(17, 2 * n)
    mk = np.zeros(n, dtype=MARKER_DTYPE)
    mk["X"] = u[0::2] ** 3 * 1.1 - 0.05
    mk["Y"] = u[1::2] * 1.02 - 0.01
    mk["X"][::997] = np.nan
    wl.markers = mk
    G = gpu.MicProblem(wl)
    O = oraclepy.OracleProblem(wl)
    assert G.findMarkerCells() == O.findMarkerCells()
    got = G.markers
    for f in ("cellX", "cellY"):
        np.testing.assert_array_equal(got[f], O.markers[f])
    np.testing.assert_array_equal(G.sorted_ids(), np.argsort(sort_keys(O.markers, wl.grid), kind="stable"))


def test_empty_marker_set():
    wl = W.convection_box(ncell=8, nm=2)
    wl.markers = wl.markers[:0]
    G = gpu.MicProblem(wl, capacity=16)
    assert G.findMarkerCells() == 0
    G.projectMarkersNodesAll2()
    assert np.all(G.get_nodal("rho") == 0.0)
    assert np.all(G.get_nodal("muS") == 1e99)
    G.step(wl.dt, wl.dt)


# ---- bit-exact build against the oracle in sorted order --------------------------------


@pytest.mark.parametrize("make", [
    lambda: transcendental_free(W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=31)),
    lambda: transcendental_free(W.convection_box(ncell=24, nm=3, seed=32)),
])
def test_exact_build_bitwise_over_steps(make):
    wl = make()
    G = gpu.MicProblem(wl, exact=True)
    S = SortedOracle(wl)
    D = wl.options.subgridStressDiffusivity
    for step in range(3):
        G.findMarkerCells()
        S.follow(G.sorted_ids())
        O = S.O
        O.findMarkerCells()
        for P in (G, O):
            P.updateMarkerRho()
            P.projectMarkersNodesAll2()
        for f in PROJECTED_FIELDS:
            ok, msg = exact(G.get_nodal(f), O.get_nodal(f))
            assert ok, "step %d proj1 %s %s" % (step, f, msg)
        assert G.checkPlasticYielding(wl.dt) == O.checkPlasticYielding(wl.dt)
        for P in (G, O):
            P.limitViscosity()
            P.projectMarkersNodesAll2()
            P.updateMarkerStrainPressure(wl.dt)
        fails = compare_markers(G.markers, S.caller_order())
        assert not fails, ("step %d strain" % step, fails)
        rg, ro = G.updateGlobalStrainRateResidual(0), O.updateGlobalStrainRateResidual(0)
        assert abs(rg - ro) <= 1e-13 * abs(ro)
        for P in (G, O):
            if D > 0:
                P.subgridStressChanges(wl.dt, D)
            P.updateMarkerStress()
            P.subgridTemperatureChanges(wl.dt_thermal)
            P.advectMarkersRK(wl.dt_thermal)
        fails = compare_markers(G.markers, S.caller_order())
        assert not fails, ("step %d end" % step, fails)
        assert G.maxAbsSxx() == O.maxAbsSxx()
        assert G.maxMarkerT() == O.maxMarkerT()


def test_exact_build_subgrid_stress_bitwise():
    """The subgrid stress gather (quadrant scatter with its double-counted half lines and the
    tent-weighted centre scatter) against the oracle in sorted order."""
    wl = W.vep_slab_box(nx_cells=24, ny_cells=8, nm=4, seed=41)
    for k in range(wl.materials.nMaterials):
        wl.materials.hasEtaT[k] = 0
    G = gpu.MicProblem(wl, exact=True)
    S = SortedOracle(wl)
    G.findMarkerCells()
    S.follow(G.sorted_ids())
    S.O.findMarkerCells()
    # geometry-independent inputs; only the exp of the relaxation factor differs by an ulp
    G.subgridStressChanges(wl.dt, 1.0)
    S.O.subgridStressChanges(wl.dt, 1.0)
    for f in ("dsxx", "dsyy", "dsxy"):
        ok, msg = close(G.get_nodal(f), S.O.get_nodal(f), 1e-13)
        assert ok, f + " " + msg
    fails = compare_markers(G.markers, S.caller_order(), fields=["sxx", "syy", "sxy"], rtol=1e-13)
    assert not fails, fails


@pytest.mark.parametrize("stag", [(-1, -1), (0, 0), (1, 1), (-1, 1), (1, 0), (0, -1)])
@pytest.mark.parametrize("method", [0, 1, 2])
def test_generic_projection_exact(stag, method):
    wl = W.vep_slab_box(nx_cells=20, ny_cells=8, nm=3, seed=5)
    G = gpu.MicProblem(wl, exact=True)
    S = SortedOracle(wl)
    G.findMarkerCells()
    S.follow(G.sorted_ids())
    S.O.findMarkerCells()
    G.projectMarkerFieldToNodes("eta", "srr", stag[0], stag[1], method)
    S.O.projectMarkerFieldToNodes("eta", "srr", stag[0], stag[1], method)
    ok, msg = exact(G.get_nodal("srr"), S.O.get_nodal("srr"))
    assert ok, msg
    mp = [3.0, 4.5]
    G.projectMarkerFieldToNodes(None, "Cp", stag[0], stag[1], method, matprop=mp)
    S.O.projectMarkerFieldToNodes(None, "Cp", stag[0], stag[1], method, matprop=np.array(mp + [0.0] * 6))
    ok, msg = exact(G.get_nodal("Cp"), S.O.get_nodal("Cp"))
    assert ok, msg


# ---- product build against the reference (golden vectors, reference marker order) ------


@pytest.mark.parametrize("exact_build", [False, True])
@pytest.mark.parametrize("name", ["convection_box_8", "vep_slab_box_16x4", "edge_cases", "periodic_box",
                                  "vep_jaumann"])
def test_sequence_matches_reference_golden(name, exact_build):
    wl, z = load_case(name)
    G = gpu.MicProblem(wl, exact=exact_build, jaumann=is_jaumann(z))
    fails = []

    def check(tag, P, nout=None, value=None):
        if tag.endswith("after_find"):
            if int(z[tag[:3] + "nout"]) != nout:
                fails.append("%s nOut" % tag)
        if tag.endswith(("proj1", "proj2")):
            for f in PROJECTED_FIELDS:
                ok, msg = close(P.get_nodal(f), z[tag + "_" + f], RTOL)
                if not ok:
                    fails.append("%s %s: %s" % (tag, f, msg))
            return
        if tag.endswith("after_subgrid_stress"):
            for f in ("dsxx", "dsyy", "dsxy"):
                ok, msg = close(P.get_nodal(f), z[tag[:3] + "ds_" + f], RTOL)
                if not ok:
                    fails.append("%s %s: %s" % (tag, f, msg))
        if value is not None:
            ok, msg = close(np.array([value]), np.array([float(z[tag])]), RTOL)
            if not ok:
                fails.append("%s %s" % (tag, msg))
            return
        for msg in compare_markers(P.markers, as_markers(z[tag]), rtol=RTOL):
            fails.append("%s %s" % (tag, msg))

    run_sequence(G, wl, z, check=check)
    assert not fails, "\n".join(fails[:25])


def test_step_equals_entry_point_sequence():
    wl = W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=51)
    A = gpu.MicProblem(wl)
    B = gpu.MicProblem(wl)
    for _ in range(2):
        _, ra = A.step(wl.dt, wl.dt_thermal)
        B.findMarkerCells()
        B.updateMarkerRho()
        B.projectMarkersNodesAll2()
        B.checkPlasticYielding(wl.dt)
        B.limitViscosity()
        B.projectMarkersNodesAll2()
        B.updateMarkerStrainPressure(wl.dt)
        rb = B.updateGlobalStrainRateResidual(0)
        B.subgridStressChanges(wl.dt, wl.options.subgridStressDiffusivity)
        B.updateMarkerStress()
        B.subgridTemperatureChanges(wl.dt_thermal)
        B.advectMarkersRK(wl.dt_thermal)
        assert ra == rb
    assert not compare_markers(A.markers, B.markers)
    for f in PROJECTED_FIELDS + ["dsxx", "dsyy", "dsxy"]:
        assert exact(A.get_nodal(f), B.get_nodal(f))[0], f


def test_deterministic_across_runs():
    wl = W.vep_slab_box(nx_cells=64, ny_cells=16, nm=4, seed=61)
    outs = []
    for _ in range(2):
        G = gpu.MicProblem(wl)
        for _ in range(2):
            G.step(wl.dt, wl.dt_thermal)
        outs.append((G.markers, {f: G.get_nodal(f) for f in PROJECTED_FIELDS}))
    assert not compare_markers(outs[0][0], outs[1][0])
    for f in PROJECTED_FIELDS:
        assert exact(outs[0][1][f], outs[1][1][f])[0], f


def test_nan_strain_rate_residual_is_an_error():
    """The reference aborts on a NaN strain-rate residual (updateMarkerStrainPressure.c:302-306);
    the library returns MIC_ERR_NAN and keeps the context usable."""
    wl = W.convection_box(ncell=8, nm=2)
    wl.markers["eta"][5] = 0.0
    wl.markers["mu"][5] = 0.0
    G = gpu.MicProblem(wl)
    G.findMarkerCells()
    with pytest.raises(gpu.MicError) as e:
        G.updateMarkerStrainPressure(wl.dt)
    assert e.value.code == 5
    assert G.status().nan_residual >= 1
    G.findMarkerCells()  # still usable


def test_rejects_unsupported_boundaries():
    """A top wall of type 2 (the reference's grids are never periodic in y) is refused with
    MIC_ERR_BC; on a grid periodic in x the routines outside the marker path (here the density
    control) return MIC_ERR_BC and leave the context usable"""
    wl = W.convection_box(ncell=8, nm=2)
    wl.bcs.mechBCTop.type[0] = 2
    with pytest.raises(gpu.MicError) as e:
        gpu.MicProblem(wl)
    assert e.value.code == 7
    from fvmic2d_gb300.mic_types import DensityOptions

    wp = W.periodic_box(nx_cells=16, ny_cells=6, nm=2, seed=5)
    G = gpu.MicProblem(wp)
    with pytest.raises(gpu.MicError) as e:
        G.checkMarkerDensity(DensityOptions(NMX=4, NMY=4, minMarkers=1, maxMarkers=100))
    assert e.value.code == 7
    assert G.findMarkerCells() == 0


# ---- full-size properties ----------------------------------------------------------------


def test_full_size_vep_box_step_matches_oracle():
    """One whole step at the 1025 x 257 / 4,194,304-marker size against the oracle in the
    reference's marker order (relative 1e-12), plus size-independent properties."""
    wl = W.vep_slab_box()
    G = gpu.MicProblem(wl)
    O = oraclepy.OracleProblem(wl)
    e, r_o = O.step(wl.dt, wl.dt_thermal)
    assert e == 0
    _, r_g = G.step(wl.dt, wl.dt_thermal)
    assert abs(r_g - r_o) <= RTOL * abs(r_o)
    got = G.markers
    fails = compare_markers(got, O.markers, rtol=RTOL)
    assert not fails, fails
    for f in PROJECTED_FIELDS + ["dsxx", "dsyy", "dsxy"]:
        ok, msg = close(G.get_nodal(f), O.get_nodal(f), RTOL)
        assert ok, f + " " + msg
    # the sort is a permutation in cell order and cell_start brackets every cell
    G.findMarkerCells()
    ids = G.sorted_ids()
    assert np.array_equal(np.sort(ids), np.arange(len(ids)))
    mk = G.markers
    keys = sort_keys(mk, wl.grid)[ids]
    assert np.all(np.diff(keys) >= 0)
    cs = G.cell_start()
    assert cs[0] == 0 and cs[-1] == len(ids) and np.all(np.diff(cs) >= 0)


def test_constant_field_reproduction_and_partition_of_unity():
    """Projecting a constant marker field returns the constant at every node with weight
    (partition of unity of the bilinear weights), at a size far beyond the oracle's reach."""
    wl = W.vep_slab_box(nx_cells=512, ny_cells=256, nm=4, seed=71)
    wl.markers["T"] = 1234.5
    wl.markers["eta"] = 3.0e21
    G = gpu.MicProblem(wl)
    G.findMarkerCells()
    G.projectMarkersNodesAll2()
    lastT = G.get_nodal("lastT")
    assert np.all(np.abs(lastT - 1234.5) <= 1e-13 * 1234.5)
    for f in ("etaS", "etaN"):
        v = G.get_nodal(f)
        nz = v != 0.0
        assert np.all(np.abs(v[nz] - 3.0e21) <= 1e-14 * 3.0e21)


def test_project_from_scalar_matches_oracle():
    """projectMarkersNodesFromScalar (markers.c:1507) of a per-marker array in caller order"""
    wl = W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=3)
    G, O = gpu.MicProblem(wl), oraclepy.OracleProblem(wl)
    G.findMarkerCells()
    O.findMarkerCells()
    v = W.splitmix64_uniform(43, len(wl.markers)) - 0.3
    G.projectMarkersNodesFromScalar(v, "lastT")
    O.projectMarkersNodesFromScalar(v, "lastT")
    ok, msg = close(G.get_nodal("lastT"), O.get_nodal("lastT"), RTOL)
    assert ok, msg


def test_short_named_creep_exports():
    """mic_creep_newton is mic_creep_solve_batch's exact mode, bit for bit"""
    wl = W.ice_creep_box(nx_cells=8, ny_cells=8, nm=2, seed=4)
    G = gpu.MicProblem(wl)
    L = G.L
    e = np.array([1e-14, 3e-12]); T = np.array([200.0, 250.0]); d = np.array([1e-3, 1e-2]); P = np.array([1e6, 2e7])
    s = np.zeros(2); it = np.zeros(2, dtype=np.int32); r = np.zeros(2)
    assert L.mic_creep_newton(G.h, *[x.ctypes.data_as(gpu._DP) for x in (e, T, d, P)], 2,
                              s.ctypes.data_as(gpu._DP), it.ctypes.data, r.ctypes.data_as(gpu._DP)) == 0
    s2, _, _, _ = G.creep_solve(e, T, d, P, mode=0)
    assert np.array_equal(s, s2)


def test_step_split_reports_max_temperature_and_yielding():
    """mic_step_pre_stokes's maximum marker temperature (formed with the density update) is the
    entry point's (mic_max_marker_T) and numpy's over the in-domain markers, some pushed out of
    the domain with the hottest temperatures; its yield flag is checkPlasticYielding's"""
    import ctypes

    wl = W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=57)
    m = wl.markers
    m["T"] = m["T"] + np.linspace(0.0, 50.0, len(m))
    out = np.arange(len(m)) % 97 == 0
    m["X"][out] = -1.0  # out of the domain, hottest markers among them
    m["T"][out] = 5.0e3
    A = gpu.MicProblem(wl)
    B = gpu.MicProblem(wl)
    isy = ctypes.c_int(-1)
    mt = ctypes.c_double(-1.0)
    assert A.L.mic_step_pre_stokes(A.h, wl.dt, ctypes.byref(isy), ctypes.byref(mt)) == 0
    B.findMarkerCells()
    B.updateMarkerRho()
    B.projectMarkersNodesAll2()
    ref_t = B.maxMarkerT()
    ref_y = B.checkPlasticYielding(wl.dt)
    inside = ~out
    assert mt.value == ref_t == float(np.max(m["T"][inside]))
    assert isy.value == ref_y
    # the rest of the step: max |sxx| formed by the advection equals mic_max_abs_sxx's
    B.limitViscosity()
    B.projectMarkersNodesAll2()
    assert A.L.mic_step_post_stokes(A.h, wl.dt, 1, None) == 0
    B.updateMarkerStrainPressure(wl.dt)
    B.updateGlobalStrainRateResidual(0)
    B.subgridStressChanges(wl.dt, wl.options.subgridStressDiffusivity)
    B.updateMarkerStress()
    mx = ctypes.c_double(-1.0)
    assert A.L.mic_step_post_thermal(A.h, wl.dt_thermal, ctypes.byref(mx)) == 0
    B.subgridTemperatureChanges(wl.dt_thermal)
    B.advectMarkersRK(wl.dt_thermal)
    assert mx.value == B.maxAbsSxx() > 0.0
    assert not compare_markers(A.markers, B.markers)


@pytest.mark.parametrize("exact_build", [False, True])
def test_residual_of_markers_not_yet_binned(exact_build):
    """updateGlobalStrainRateResidual called on markers just uploaded in the caller's order (the
    binning it triggers re-sorts the columns): the residual of the sorted strain-rate residuals,
    the same as from markers already binned, and the oracle's"""
    wl = W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=5)
    G = gpu.MicProblem(wl, exact=exact_build)
    O = oraclepy.OracleProblem(wl)
    for P in (G, O):
        P.findMarkerCells()
        P.updateMarkerRho()
        P.projectMarkersNodesAll2()
        P.updateMarkerStrainPressure(wl.dt)
    r_bin = G.updateGlobalStrainRateResidual(0)
    r_o = O.updateGlobalStrainRateResidual(0)
    G.upload_markers(G.markers)  # caller order, no binning yet
    r_up = G.updateGlobalStrainRateResidual(1)
    assert r_up == r_bin
    ok, msg = close([r_up], [r_o], RTOL)
    assert ok, msg


@pytest.mark.parametrize("exact_build", [False, True])
def test_periodic_step_equals_entry_points_and_wraps(exact_build):
    """On a grid periodic in x (mechBCLeft/Right vx type 2) mic_step gives the entry-point
    sequence's markers and nodal fields bit for bit, markers leaving through x = LX come back
    near x = 0 (markers.c:2225-2231), and every marker stays in the domain"""
    wl = W.periodic_box(nx_cells=24, ny_cells=8, nm=4, seed=21)
    A = gpu.MicProblem(wl, exact=exact_build)
    B = gpu.MicProblem(wl, exact=exact_build)
    x0 = A.markers["X"].copy()
    for _ in range(3):
        _, ra = A.step(wl.dt, wl.dt_thermal)
        assert B.findMarkerCells() == 0
        B.updateMarkerRho()
        B.projectMarkersNodesAll2()
        B.checkPlasticYielding(wl.dt)
        B.limitViscosity()
        B.projectMarkersNodesAll2()
        B.updateMarkerStrainPressure(wl.dt)
        rb = B.updateGlobalStrainRateResidual(0)
        B.subgridStressChanges(wl.dt, wl.options.subgridStressDiffusivity)
        B.updateMarkerStress()
        B.subgridTemperatureChanges(wl.dt_thermal)
        B.advectMarkersRK(wl.dt_thermal)
        if exact_build:
            assert ra == rb
    ma, mb = A.markers, B.markers
    if exact_build:
        assert not compare_markers(ma, mb)
        for f in PROJECTED_FIELDS + ["dsxx", "dsyy", "dsxy"]:
            assert exact(A.get_nodal(f), B.get_nodal(f))[0], f
    else:  # the step reuses values across passes (rounding at the last place)
        assert not compare_markers(ma, mb, rtol=1e-12)
    X = ma["X"]
    assert np.all((X >= 0.0) & (X <= wl.grid.LX))
    assert np.any((x0 > 0.9 * wl.grid.LX) & (X < 0.1 * wl.grid.LX))  # crossed the seam
    assert A.findMarkerCells() == 0
