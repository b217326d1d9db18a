"""The periodic-x golden fixture (tests/golden/periodic_box.npz, made by make_golden.py from the
reference's own sources with gridGenerator.c's periodic set-up) is what it claims to be: the
reference binned markers into NX cells in x, projected onto NX node columns, and wrapped markers
that left through x = LX back into the domain (markers.c:2225-2231)."""
import os

import numpy as np

from fvmic2d_gb300 import workloads as W
from fvmic2d_gb300.mic_types import BCs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_periodic_fixture_is_periodic():
    z = np.load(os.path.join(GOLDEN, "periodic_box.npz"))
    x, LX = z["x"], float(z["LX"])
    NX = len(x)
    # NX lines of the NX + 1 uniform ones from 0 to LX: line NX is LX itself
    np.testing.assert_array_equal(x, W.spacing_uniform(0.0, LX, NX + 1)[:NX])
    bcs = BCs.from_buffer_copy(z["bcs_bytes"].tobytes())
    assert bcs.mechBCLeft.type[0] == 2 and bcs.mechBCRight.type[0] == 2  # nodalFields.c:12
    crossed = 0
    for s in range(3):
        found = z["s%d_after_find" % s]
        assert int(z["s%d_nout" % s]) == 0
        assert found["cellX"].max() == NX - 1  # the periodic grid's last cell
        after = z["s%d_after_advect" % s]
        assert np.all((after["X"] >= 0.0) & (after["X"] <= LX))
        crossed += int(np.sum((found["X"] > 0.9 * LX) & (after["X"] < 0.1 * LX)))
        for f in ("rho", "etaN", "soxx"):
            assert z["s%d_proj1_%s" % (s, f)].shape == (len(z["y"]), NX)
    assert crossed > 0
    # nodes on the seam receive the last cell's markers: column 0 sums both sides of x = 0
    assert np.all(z["s0_proj1_rho"][:, 0] != 0.0)
