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
from tests.timestep_case import timestep_case

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
def test_timestep_matches_reference(build):
    z = np.load(os.path.join(GOLDEN, "subduction_step.npz"))
    wl, topt = timestep_case()
    wl.markers = z["before"].view(MARKER_DTYPE).copy()
    ref = z["after"].view(MARKER_DTYPE)
    G = gpu.MicProblem(wl, exact=(build == "exact"))
    rep = G.subductionTimestep(topt, 0.0)
    assert rep["stopped"] == 0
    for k in ("plastic_iterations", "is_yielding", "converged", "thermal_resolves"):
        assert rep[k] == int(z["rep_" + k]), k
    for k in ("dt", "displacement_dt", "Kbond", "Kcont", "max_T", "max_temp_change", "max_abs_sxx"):
        assert abs(rep[k] - float(z["rep_" + k])) <= 1e-9 * abs(float(z["rep_" + k])), (k, rep[k], z["rep_" + k])
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
        a, b = G.get_nodal(f), z["nodal_" + f]
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b)), f
