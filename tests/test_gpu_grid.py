"""GPU grid routines between the solves (nodalStressStrain, limitDisplacementTimestep,
retrieveSolutions) against the reference's own outputs: bit-exact in both builds (the grid
kernels evaluate every operation as an IEEE intrinsic in the reference's order)."""
import os

import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from tests.helpers import exact
from tests.test_oracle_pin import GRID_OUT, grid_case, grid_case_from_golden

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("build", ["exact", "product"])
@pytest.mark.parametrize("kind", ["free_slip", "prescribed"])
def test_grid_routines_match_reference_outputs(kind, build):
    z = np.load(os.path.join(GOLDEN, "grid_routines.npz"))
    wl, S = grid_case_from_golden(z, kind)
    G = gpu.MicProblem(wl, exact=(build == "exact"))
    G.nodalStressStrain(3.0e11)
    for name in GRID_OUT:
        ref = z["%s_out_%s" % (kind, name)]
        ok, msg = exact(G.get_nodal(name), ref)
        assert ok, (name, msg)
    dts = [G.limitDisplacementTimestep(1e14, 0.5), G.limitDisplacementTimestep(1e30, 0.1)]
    assert np.array_equal(np.array(dts), z[kind + "_dt"])
    assert G.retrieveSolutions(z[kind + "_S"], 1e20) == 0
    for name in ("vx", "vy", "p"):
        ok, msg = exact(G.get_nodal(name), z["%s_ret_%s" % (kind, name)])
        assert ok, (name, msg)


def test_time_step_edge_cases():
    """no moving node and no density change: the limit is the input; NaN velocities are skipped"""
    wl, _ = grid_case("free_slip", 5)
    G = gpu.MicProblem(wl)
    for f in ("vx", "vy", "rhodot"):
        G.set_nodal(f, np.zeros((wl.grid.NY, wl.grid.NX)))
    assert G.limitDisplacementTimestep(123.0, 0.5) == 123.0
    vx = np.zeros((wl.grid.NY, wl.grid.NX))
    vx[2, 3] = np.nan
    vx[4, 5] = 1e-3
    G.set_nodal("vx", vx)
    dx = min(wl.grid.x[6] - wl.grid.x[5], wl.grid.x[5] - wl.grid.x[4])
    assert G.limitDisplacementTimestep(1e30, 0.5) == dx / 1e-3 * 0.5
