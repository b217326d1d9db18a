"""mic_autotune: per-kernel launch block sizes measured on the context's own workload.  Tuning
leaves the marker columns and nodal fields exactly as they were, the sizes it picks are among the
candidates, and steps run with tuned sizes give the results of steps run with the default size,
bit for bit (every tuned kernel is one thread per marker)."""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from fvmic2d_gb300 import workloads as W
from fvmic2d_gb300.mic_types import MARKER_DTYPE, NF

pytestmark = pytest.mark.gpu


def _state(P):
    m = P.markers
    return np.array(m, copy=True), {f: P.get_nodal(f).copy() for f in NF}


def test_autotune_keeps_state_and_results():
    wl = W.vep_slab_box(nx_cells=96, ny_cells=24, nm=4, seed=7)
    A = gpu.MicProblem(wl)
    B = gpu.MicProblem(wl)
    A.step(wl.dt, wl.dt)  # tune from a mid-run state: sorted columns, projected fields
    B.step(wl.dt, wl.dt)
    before_m, before_n = _state(A)
    chosen = A.autotune(wl.dt, wl.dt, subgrid_stress=1, steps=2)
    assert set(chosen) == set(gpu.TUNE_KERNELS)
    assert all(b in (128, 256, 512) for b in chosen.values()), chosen
    assert A.tuning() == chosen
    after_m, after_n = _state(A)
    assert after_m.tobytes() == before_m.tobytes()
    for f in NF:
        assert np.array_equal(after_n[f], before_n[f]), f
    for _ in range(2):
        A.step(wl.dt, wl.dt)
        B.step(wl.dt, wl.dt)
    a, b = A.markers, B.markers
    assert a.tobytes() == b.tobytes()
    for f in ("vx", "rho", "etaN", "soxy", "lastT"):
        assert np.array_equal(A.get_nodal(f), B.get_nodal(f)), f


def test_tuning_can_be_set_and_is_checked():
    wl = W.vep_slab_box(nx_cells=32, ny_cells=8, nm=4, seed=2)
    A = gpu.MicProblem(wl)
    A.set_tuning({"k_advect": 512, "k_yield": 128})
    t = A.tuning()
    assert t["k_advect"] == 512 and t["k_yield"] == 128 and t["k_reorder"] == 256
    with pytest.raises(gpu.MicError):
        A.set_tuning({"k_advect": 384})
    B = gpu.MicProblem(wl)
    A.step(wl.dt, wl.dt)
    B.step(wl.dt, wl.dt)
    assert A.markers.tobytes() == B.markers.tobytes()
    assert MARKER_DTYPE.itemsize == A.markers.dtype.itemsize
