"""The reference-side binding on the GPU: fvmic2d's routines called by their own names and
signatures (fvmic2d_gb300/refglue/fvmic2d_glue.c, driven by tests/refglue/glue_driver.c on a
MarkerSet and petsc_lite Vecs) give the reference's results.

* The recorded entry-point sequences of the three golden cases (outputs of the reference's own
  compiled routines): within 1e-12 (product and FMA-free builds of the library).
* The set-up of main_subduction.c: allocateMarkers, resetMarkers, distributeMarkersUniformInDomain,
  host-side initial conditions written into MarkerSet.markers, then steps -- against the oracle
  doing the same on its own array.
* checkMarkerDensity against the reference's outputs; the residual routines of residual.h.
"""
import os

import numpy as np
import pytest

from fvmic2d_gb300 import workloads as W
from fvmic2d_gb300.mic_types import MARKER_DTYPE, PROJECTED_FIELDS, DensityOptions
from oracle import oraclepy
from tests.helpers import RTOL, close, compare_markers
from tests.refglue import gluepy
from tests.test_gpu_density import _split_compare
from tests.test_oracle_pin import as_markers, load_case, run_sequence

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("exact_build", [False, True])
@pytest.mark.parametrize("name", ["convection_box_8", "vep_slab_box_16x4", "edge_cases"])
def test_binding_sequence_matches_reference_golden(name, exact_build):
    wl, z = load_case(name)
    P = gluepy.GlueProblem(wl, exact=exact_build)
    fails = []

    def check(tag, Q, nout=None, value=None):
        if tag.endswith("after_find"):
            if int(z[tag[:3] + "nout"]) != nout:
                fails.append("%s nOut %s" % (tag, nout))
        if tag.endswith(("proj1", "proj2")):
            for f in PROJECTED_FIELDS:
                ok, msg = close(Q.get_nodal(f), z[tag + "_" + f], RTOL)
                if not ok:
                    fails.append("%s %s: %s" % (tag, f, msg))
            return
        if tag.endswith("after_subgrid_stress"):
            for f in ("dsxx", "dsyy", "dsxy"):
                ok, msg = close(Q.get_nodal(f), z[tag[:3] + "ds_" + f], RTOL)
                if not ok:
                    fails.append("%s %s: %s" % (tag, f, msg))
        if value is not None:
            ok, msg = close(np.array([value]), np.array([float(z[tag])]), RTOL)
            if not ok:
                fails.append("%s %s" % (tag, msg))
            return
        for msg in compare_markers(Q.markers, as_markers(z[tag]), rtol=RTOL):
            fails.append("%s %s" % (tag, msg))

    try:
        run_sequence(P, wl, z, check=check)
    finally:
        P.close()
    assert not fails, "\n".join(fails[:25])


def _host_initial_conditions(mk, wl):
    """what fvmic2d's initial-condition routine does on the host array after distribution: the
    material, the temperature field and the viscosity of the convection box"""
    mk["Mat"] = 0
    mk["T"] = 1.0 - mk["Y"] + 0.01 * np.cos(np.pi * mk["X"]) * np.sin(np.pi * mk["Y"])
    mk["mu"] = wl.materials.materialMu[0]
    mk["eta"] = wl.materials.materialEta[0] * np.exp(-wl.materials.QonR[0] * mk["T"])


def test_binding_setup_and_steps_match_oracle():
    wl = W.convection_box(ncell=16, nm=4, seed=3)
    cap = 4 * 4 * 16 * 16 + 64
    P = gluepy.GlueProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE), capacity=cap)
    O = oraclepy.OracleProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE))
    try:
        P.resetMarkers()
        n = P.distributeMarkersUniformInDomain(4, 4)
        mk_o, n_o = O.distribute_uniform(4, 4, seed=0, cap=cap)
        assert n == n_o
        got = P.markers  # the host array is current after distribution
        assert np.array_equal(got.view(np.uint8), mk_o[:n].view(np.uint8))
        # host-side initial conditions, written into MarkerSet.markers by host code
        mk = got.copy()
        _host_initial_conditions(mk, wl)
        assert P.L.gd_set_markers(P.h, mk.ctypes.data, n) == 0
        O.markers = mk.copy()
        D = wl.options.subgridStressDiffusivity
        for step in range(2):
            for Q in (P, O):
                Q.findMarkerCells()
                Q.updateMarkerRho()
                Q.projectMarkersNodesAll2()
                Q.checkPlasticYielding(wl.dt)
                Q.limitViscosity()
                Q.projectMarkersNodesAll2()
                Q.updateMarkerStrainPressure(wl.dt)
            for f in PROJECTED_FIELDS:
                ok, msg = close(P.get_nodal(f), O.get_nodal(f), RTOL)
                assert ok, (step, f, msg)
            rp, ro = P.updateGlobalStrainRateResidual(step), O.updateGlobalStrainRateResidual(step)
            ok, msg = close([rp], [ro], RTOL)
            assert ok, msg
            for Q in (P, O):
                if D > 0:
                    Q.subgridStressChanges(wl.dt, D)
                Q.updateMarkerStress()
                Q.subgridTemperatureChanges(wl.dt_thermal)
                Q.advectMarkersRK(wl.dt_thermal)
            fails = compare_markers(P.markers, O.markers, rtol=RTOL)
            assert not fails, (step, fails)
        # residual.h: stored residuals and the convergence test over them
        P.setGlobalStrainRateResidual(5, 2.0)
        P.setGlobalStrainRateResidual(6, 2.0 * (1 + 1e-9))
        assert P.checkConvergence(1e-30, 1e-6, 6) == 2
        assert P.checkConvergence(3.0, 1e-12, 6) == 1
        assert P.checkConvergence(1e-30, 1e-12, 6) == 0
    finally:
        P.close()


def test_binding_marker_density_matches_reference_outputs():
    z = np.load(os.path.join(GOLDEN, "marker_density.npz"))
    wl, _ = W.density_case()
    before = z["seed1_before"].view(MARKER_DTYPE).ravel().copy()
    ref = z["seed1_after"].view(MARKER_DTYPE).ravel()
    dopt = DensityOptions.from_buffer_copy(z["options_bytes"].tobytes())
    # the drand48 stream the binding's context starts from is srand48(1), main's seed
    P = gluepy.GlueProblem(wl, markers=before, capacity=int(z["seed1_cap"]))
    try:
        P.findMarkerCells()
        n = P.checkMarkerDensity(dopt)
        got = P.markers
        assert n == len(ref)
        ok, msg = _split_compare(got, ref, z["seed1_special"])
        assert ok, msg
    finally:
        P.close()
