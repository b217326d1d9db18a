"""Parity at the benchmark configurations' own sizes and step counts, after every step: the
CUDA path (product build, through the C ABI) against the CPU oracle in the reference's marker
order, relative 1e-12 with the absolute floor of tests/helpers.py.

* convection box, 64 x 64 cells, 65,536 markers: all 10 steps;
* visco-elasto-plastic box, 1025 x 257 nodes, 4,194,304 markers: 3 consecutive steps;
* composite ice creep box, 1025 x 1025 nodes, 16,777,216 markers: the law-7 yield pass on every
  marker, against the oracle's solve on a strided subset (every 61st marker), exact and surrogate;
* convection ensemble: two of its members stepped inside a captured ensemble graph against the
  oracle stepping each alone.
"""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from fvmic2d_gb300.mic_types import PROJECTED_FIELDS
from oracle import oraclepy
from tests.helpers import RTOL, close, compare_markers

pytestmark = pytest.mark.gpu


def _check_state(G, O, what, nodal=PROJECTED_FIELDS):
    fails = compare_markers(G.markers, O.markers, rtol=RTOL)
    assert not fails, (what, fails)
    for f in nodal:
        ok, msg = close(G.get_nodal(f), O.get_nodal(f), RTOL)
        assert ok, (what, f, msg)


def _step_both(G, O, wl, k):
    e, r_o = O.step(wl.dt, wl.dt_thermal)
    assert e == 0
    _, r_g = G.step(wl.dt, wl.dt_thermal)
    ok, msg = close([r_g], [r_o], RTOL)
    assert ok, ("residual", k, msg)


def test_convection_box_all_ten_steps():
    wl = W.convection_box()
    assert len(wl.markers) == 65536 and (wl.grid.NX, wl.grid.NY) == (65, 65)
    G = gpu.MicProblem(wl)
    O = oraclepy.OracleProblem(wl)
    for k in range(10):
        _step_both(G, O, wl, k)
        _check_state(G, O, "step %d" % (k + 1))
    G.close()


def test_vep_box_full_size_three_steps():
    wl = W.vep_slab_box()
    assert len(wl.markers) == 4194304
    G = gpu.MicProblem(wl)
    O = oraclepy.OracleProblem(wl)
    for k in range(3):
        _step_both(G, O, wl, k)
        _check_state(G, O, "step %d" % (k + 1), nodal=PROJECTED_FIELDS + ["dsxx", "dsyy", "dsxy"])
    G.close()


def test_ice_box_full_size_law7_pass():
    """checkPlasticYielding with the composite creep law on all 16,777,216 markers: the exact
    solve within 1e-12 of the oracle's, and the tensor-core surrogate with FP64 polish within
    1e-6 in stress (eta = s* / (2 edot)), on every 61st marker; the rest of the markers
    untouched but for viscosity and modulus"""
    wl = W.ice_creep_box()
    G = gpu.MicProblem(wl)
    G.set_grain_size(wl.grain_size)
    sub = np.arange(0, len(wl.markers), 61)
    O = oraclepy.OracleProblem(wl, markers=wl.markers[sub].copy())
    O.set_grain_size(wl.grain_size[sub])
    O.findMarkerCells()
    O.checkPlasticYielding(wl.dt)
    G.findMarkerCells()
    G.creep_configure(mode=0, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    G.checkPlasticYielding(wl.dt)
    got = G.markers
    fails = compare_markers(got[sub], O.markers, rtol=RTOL)
    assert not fails, fails
    st = G.creep_stats()
    assert st["markers"] == len(wl.markers) and st["max_residual"] <= 2e-14
    for f in ("X", "Y", "T", "sxx", "exx", "p"):
        assert np.array_equal(got[f], wl.markers[f]), f
    # the surrogate path, polished to a rate residual of 1e-7
    G.creep_train()
    G.creep_configure(mode=2, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    G.checkPlasticYielding(wl.dt)
    eta2 = G.markers["eta"]
    rel = np.abs(eta2[sub] / O.markers["eta"] - 1.0)
    assert rel.max() <= 1e-6, rel.max()
    st = G.creep_stats()
    assert st["tc_timeouts"] == 0 and st["max_residual"] <= 1e-7
    assert st["fallbacks"] <= 1e-3 * len(wl.markers)
    G.close()


def test_two_ensemble_members_against_oracle():
    wls = W.convection_ensemble()
    order = sorted(range(len(wls)), key=lambda i: (wls[i].grid.NX - 1) * (wls[i].grid.NY - 1) * wls[i].nm[0] ** 2)
    pick = [wls[order[0]], wls[order[len(order) // 4]]]
    members = []
    for wl in pick:
        P = gpu.MicProblem(wl, capacity=wl.capacity)
        gpu.initialize_markers(P, *wl.nm, seed=wl.seed)
        members.append(P)
    oracles = [oraclepy.OracleProblem(wl, markers=P.markers) for wl, P in zip(pick, members)]
    for P, O in zip(members, oracles):  # the initial nodal state the step starts from
        for f in ("lastT",):
            O.set_nodal(f, P.get_nodal(f))
    E = gpu.MicEnsemble(members)
    dts = np.array([wl.dt for wl in pick])
    for k in range(3):
        E.step(dts, dts, subgrid_stress=1, graph=True)
        E.synchronize()
        for P, O, wl in zip(members, oracles, pick):
            e, _ = O.step(wl.dt, wl.dt, True)
            assert e == 0
            _check_state(P, O, "member %dx%d step %d" % (wl.grid.NX - 1, wl.grid.NY - 1, k + 1))
    E.close()
    for P in members:
        P.close()
