"""GPU marker checkpoints in the reference's binary format: the file written from the device
columns is byte-identical to the reference's saveMarkersBinary, and restarting from it gives the
reference's restartFromMarkers markers (also from a binned, reordered marker set)."""
import os

import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from fvmic2d_gb300.mic_types import MARKER_DTYPE
from tests.helpers import same_fields

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("binned", [False, True])
def test_checkpoint_matches_reference_outputs(tmp_path, binned):
    z = np.load(os.path.join(GOLDEN, "marker_checkpoint.npz"))
    wl = W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=2)
    before = z["markers_in"].view(MARKER_DTYPE).ravel().copy()
    G = gpu.MicProblem(wl, markers=before, capacity=len(before) + 10)
    if binned:  # columns in cell order: the file still lists markers in the caller's order
        G.findMarkerCells()
        G.projectMarkersNodesAll2()
    path = str(tmp_path / "Markers.0.7")
    G.saveMarkersBinary(path, 1.25e13)
    assert np.array_equal(np.fromfile(path, dtype=np.uint8), z["file_bytes"])
    R = gpu.MicProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE), capacity=len(before) + 10)
    assert R.restartFromMarkers(path) == float(z["elapsed"])
    ok, msg = same_fields(R.markers, z["restart"].view(MARKER_DTYPE).ravel())
    assert ok, msg


def test_restart_capacity_and_missing_file(tmp_path):
    z = np.load(os.path.join(GOLDEN, "marker_checkpoint.npz"))
    wl = W.vep_slab_box(nx_cells=16, ny_cells=4, nm=4, seed=2)
    path = str(tmp_path / "f")
    z["file_bytes"].tofile(path)
    small = gpu.MicProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE), capacity=10)
    with pytest.raises(gpu.MicError) as e:
        small.restartFromMarkers(path)
    assert e.value.code == 8  # MIC_ERR_CAPACITY
    with pytest.raises(gpu.MicError) as e:
        small.restartFromMarkers(str(tmp_path / "absent"))
    assert e.value.code == 11  # MIC_ERR_IO
