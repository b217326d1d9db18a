"""mic_nodal_upload_many / mic_nodal_download_many: several nodal fields per call.  Pinned host
buffers go through one kernel reading and writing host memory directly; pageable ones through
one copy per field; both give the per-field calls' bytes."""
import ctypes

import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from fvmic2d_gb300 import workloads as W
from fvmic2d_gb300.mic_types import NF

pytestmark = pytest.mark.gpu

UP = ["vx", "vy", "p", "soxx", "dsxy"]
DOWN = ["rho", "etaN", "soxy", "lastT"]


def _pinned(P, n):
    p = ctypes.c_void_p()
    assert P.L.mic_host_alloc(ctypes.byref(p), n * 8) == 0
    return p, np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(n,))


@pytest.mark.parametrize("pinned", [True, False])
def test_batched_transfers_match_per_field(pinned):
    wl = W.vep_slab_box(nx_cells=48, ny_cells=12, nm=4, seed=5)
    P = gpu.MicProblem(wl)
    nn = P.NX * P.NY
    rng = np.random.default_rng(3)
    src = {f: rng.standard_normal(nn) for f in UP}
    keep = []
    if pinned:
        ups = []
        for f in UP:
            p, a = _pinned(P, nn)
            a[:] = src[f]
            ups.append(p.value)
            keep.append(p)
    else:
        arrs = [np.ascontiguousarray(src[f]) for f in UP]
        ups = [a.ctypes.data for a in arrs]
    P.profile_enable(64)
    fids = (ctypes.c_int * len(UP))(*[NF[f] for f in UP])
    assert P.L.mic_nodal_upload_many(P.h, fids, (ctypes.c_void_p * len(UP))(*ups), len(UP)) == 0
    for f in UP:
        assert np.array_equal(P.get_nodal(f).ravel(), src[f]), f
    P.step(wl.dt, wl.dt)  # projected fields to read back
    if pinned:
        downs = []
        views = []
        for _ in DOWN:
            p, a = _pinned(P, nn)
            downs.append(p.value)
            views.append(a)
            keep.append(p)
    else:
        views = [np.empty(nn) for _ in DOWN]
        downs = [a.ctypes.data for a in views]
    dids = (ctypes.c_int * len(DOWN))(*[NF[f] for f in DOWN])
    assert P.L.mic_nodal_download_many(P.h, dids, (ctypes.c_void_p * len(DOWN))(*downs), len(DOWN)) == 0
    for f, a in zip(DOWN, views):
        assert np.array_equal(a, P.get_nodal(f).ravel()), f
    kernels = P.profile_read()
    P.profile_enable(0)
    assert (("k_nodal_batch_up" in kernels) and ("k_nodal_batch_down" in kernels)) == pinned, kernels.keys()
    bad = (ctypes.c_int * 1)(99)
    assert P.L.mic_nodal_upload_many(P.h, bad, (ctypes.c_void_p * 1)(ups[0]), 1) != 0
    for p in keep:
        P.L.mic_host_free(p)
    P.close()
