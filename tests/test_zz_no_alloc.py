"""Binning without allocation: mic_bin_sort_noalloc checked against the context entry point.

Some callers of this library cannot call cudaMalloc: a host that forbids device allocation
once it has started, or a plug-in whose application owns the allocator.  For them
mic_bin_sort_noalloc bins markers and returns their stable cell order using only the
caller's device buffers and a fixed scratch array inside the library.  Its results must
equal what mic_find_marker_cells (a context's binning and stable counting sort) produces
for the same markers -- exactly, since this is integer work -- on consecutive calls that
reuse the shared scratch array.

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(L, torch, grid, X, Y):
    n = len(X)
    dev = torch.device("cuda", 0)
    dX = torch.as_tensor(np.ascontiguousarray(X, dtype=np.float64), device=dev)
    dY = torch.as_tensor(np.ascontiguousarray(Y, dtype=np.float64), device=dev)
    dx = torch.as_tensor(grid.x, device=dev)
    dy = torch.as_tensor(grid.y, device=dev)
    cellX = torch.full((n,), -7, dtype=torch.int32, device=dev)
    cellY = torch.full((n,), -7, dtype=torch.int32, device=dev)
    perm = torch.full((n,), -7, dtype=torch.int32, device=dev)
    cs = torch.full((grid.ncells + 2,), -7, dtype=torch.int32, device=dev)
    nout = ctypes.c_int64(-1)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = L.mic_bin_sort_noalloc(dX.data_ptr(), dY.data_ptr(), n, dx.data_ptr(), dy.data_ptr(), grid.NX, grid.NY,
                                grid.LX, grid.LY, cellX.data_ptr(), cellY.data_ptr(), perm.data_ptr(), cs.data_ptr(),
                                stream, ctypes.byref(nout))
    assert rc == 0, L.mic_error_string(rc)
    torch.cuda.synchronize(dev)
    return cellX.cpu().numpy(), cellY.cpu().numpy(), perm.cpu().numpy(), cs.cpu().numpy(), nout.value


def _context(wl):
    G = gpu.MicProblem(wl)
    nout = G.findMarkerCells()
    mk = G.markers
    out = mk["cellX"].copy(), mk["cellY"].copy(), G.sorted_ids(), G.cell_start(), nout
    G.close()
    return out


def _workloads():
    # 16,384 cells (two radix passes) then 90,000 cells (three passes): both ping-pong orders
    a = W.vep_slab_box(nx_cells=256, ny_cells=64, nm=4, seed=81)
    b = W.convection_box(ncell=300, nm=2, seed=82)
    mk = b.markers
    u = W.splitmix64_uniform(83, len(mk))
    mk["X"] = mk["X"] + (u - 0.5) * 0.01   # some markers leave the domain
    mk["Y"][::1009] = np.nan
    return [a, b]


def test_noalloc_sort_matches_context_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    L = gpu.load()
    for wl in _workloads():
        got = _noalloc(L, torch, wl.grid, wl.markers["X"], wl.markers["Y"])
        want = _context(wl)
        for name, g, w in zip(("cellX", "cellY", "perm", "cell_start"), got[:4], want[:4]):
            np.testing.assert_array_equal(g, w, err_msg=name)
        assert got[4] == want[4]


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    L = gpu.load()
    wl = W.convection_box(ncell=8, nm=2)
    g = wl.grid
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    ibuf = torch.zeros(16, dtype=torch.int32, device=dev)
    p = buf.data_ptr()
    q = ibuf.data_ptr()
    # more markers than the fixed scratch holds: refused before any device work
    rc = L.mic_bin_sort_noalloc(p, p, gpu.NOALLOC_MAX_MARKERS + 1, p, p, g.NX, g.NY, g.LX, g.LY, q, q, q, q,
                                None, None)
    assert rc == 8  # MIC_ERR_CAPACITY
    # a grid with more cells than the histogram bound
    rc = L.mic_bin_sort_noalloc(p, p, 4, p, p, 2049, 1025, 1.0, 1.0, q, q, q, q, None, None)
    assert rc == 8
