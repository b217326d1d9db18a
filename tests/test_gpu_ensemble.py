"""GPU checks of the marker lifecycle (resetMarkers, distributeMarkersUniformInDomain) against
the oracle, and of ensembles: stepping members together -- on their own streams or as captured
CUDA graphs -- gives exactly what stepping each member alone gives."""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from fvmic2d_gb300.mic_types import MARKER_DTYPE
from oracle import oraclepy

pytestmark = pytest.mark.gpu


def _bytes(a):
    return np.ascontiguousarray(a).view(np.uint8).reshape(len(a), -1)


@pytest.mark.parametrize("case", ["uniform", "refined"])
@pytest.mark.parametrize("nm,seed", [((4, 4), 0), ((3, 5), 0), ((5, 2), 12345)])
def test_distribute_matches_oracle(case, nm, seed):
    wl = W.convection_box(ncell=8, nm=4, seed=1) if case == "uniform" else W.vep_slab_box(16, 4, nm=4, seed=2)
    cap = nm[0] * nm[1] * (wl.grid.NX - 1) * (wl.grid.NY - 1) + 40
    G = gpu.MicProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE), capacity=cap)
    G.resetMarkers()
    n = G.distributeMarkersUniformInDomain(nm[0], nm[1], seed)
    O = oraclepy.OracleProblem(wl, markers=np.zeros(0, dtype=MARKER_DTYPE))
    mk, no = O.distribute_uniform(nm[0], nm[1], seed=seed, cap=cap)
    assert n == no
    assert np.array_equal(_bytes(G.markers), _bytes(mk[:n]))


def test_distribute_keeps_other_fields_in_caller_order():
    """Without a reset the reference overwrites X, Y only: the other fields of array slot k stay
    -- also after the device has binned and reordered the markers."""
    wl = W.vep_slab_box(16, 4, nm=4, seed=2)
    G = gpu.MicProblem(wl)
    G.findMarkerCells()
    G.projectMarkersNodesAll2()  # columns now in cell order
    n = G.distributeMarkersUniformInDomain(3, 3, 7)
    O = oraclepy.OracleProblem(wl)
    mk = O.markers.copy()
    o = oraclepy.lib().orc_distribute_uniform(O.h, mk.ctypes.data, len(mk), 3, 3, 7)
    assert n == o
    got = G.markers
    G.findMarkerCells()
    exp = mk[:n].copy()
    for f in ("X", "Y", "T", "eta", "Mat", "p"):
        assert np.array_equal(got[f], exp[f]), f


def _members(seed):
    specs = [(16, 3, 1e4, 10.0), (32, 4, 3e5, 1e3), (24, 5, 1e7, 1e5), (16, 4, 2e6, 50.0)]
    return [W.convection_member(c, c, m, m, Ra, k, seed + i) for i, (c, m, Ra, k) in enumerate(specs)]


def _setup(wls):
    out = []
    for wl in wls:
        P = gpu.MicProblem(wl, capacity=wl.capacity)
        gpu.initialize_markers(P, *wl.nm, seed=wl.seed)
        out.append(P)
    return out


# (groups, tile_mult, persistent, walk): per-member kernels on member streams, and batched
# marker passes with one block per tile, a persistent round-robin walk, persistent contiguous
# runs of two tile sizes, tiles taken from a shared counter, and the members dealt to two and
# three batch groups
SCHEDULES = {
    "per_member": (0, 4, True, True),
    "tile_per_block": (1, 1, False, False),
    "round_robin": (1, 4, True, False),
    "runs": (1, 4, True, True),
    "runs16": (1, 16, True, True),
    "counter": (1, 4, True, 2),
    "two_groups": (2, 4, True, True),
    "three_groups": (3, 1, False, False),
}


@pytest.mark.parametrize("schedule", list(SCHEDULES))
@pytest.mark.parametrize("graph", [True, False])
def test_ensemble_matches_members_stepped_alone(graph, schedule):
    wls = _members(40)
    A = _setup(wls)
    B = _setup(wls)
    E = gpu.MicEnsemble(A)
    E.set_schedule(*SCHEDULES[schedule])
    assert E.schedule()["groups"] == SCHEDULES[schedule][0]
    dts = np.array([wl.dt for wl in wls])

    def compare():
        E.synchronize()
        for a, b in zip(A, B):
            assert a.n == b.n
            assert np.array_equal(_bytes(a.markers), _bytes(b.markers))
            for f in ("rho", "etaN", "etaS", "lastT"):
                assert np.array_equal(a.get_nodal(f), b.get_nodal(f)), f

    for step in range(4):
        E.step(dts, dts, subgrid_stress=1, graph=graph)
        for b, dt in zip(B, dts):
            b.step(dt, dt, True)
        if step in (0, 3):
            compare()
    # new time steps and a changed member force a fresh capture
    dts = dts * 0.75
    A[1].wl.materials.QonR[0] *= 1.5
    for P in (A[1], B[1]):
        P._check(P.L.mic_set_materials(P.h, gpu.ctypes.byref(A[1].wl.materials)), "mic_set_materials")
    for step in range(3):
        E.step(dts, dts, subgrid_stress=1, graph=graph)
        for b, dt in zip(B, dts):
            b.step(dt, dt, True)
    compare()
    launches, per_graph = E.launch_count()
    assert launches > 0
    if graph and SCHEDULES[schedule][0] == 0:
        assert per_graph >= 25 * len(A)
    E.close()


def test_ensemble_autotune_keeps_states_and_results():
    """mic_ensemble_autotune tunes every member and picks an issue order by timing graph replays
    from saved states: the members' states are those from before the call, and stepping on gives
    the members' results stepped alone, bit for bit"""
    wls = _members(40)
    A = _setup(wls)
    B = _setup(wls)
    E = gpu.MicEnsemble(A)
    dts = np.array([wl.dt for wl in wls])
    E.step(dts, dts, subgrid_stress=1, graph=True)
    for b, dt in zip(B, dts):
        b.step(dt, dt, True)
    E.synchronize()
    before = [_bytes(a.markers) for a in A]
    order = E.autotune(dts, dts, subgrid_stress=1, steps=1)
    assert sorted(order) == list(range(len(A)))
    sch = E.schedule()
    assert sch["tile_mult"] in (1, 4) and 0 <= sch["groups"] <= 8
    for a, m in zip(A, before):
        assert np.array_equal(_bytes(a.markers), m)
    for _ in range(3):
        E.step(dts, dts, subgrid_stress=1, graph=True)
        for b, dt in zip(B, dts):
            b.step(dt, dt, True)
    E.synchronize()
    for a, b in zip(A, B):
        assert np.array_equal(_bytes(a.markers), _bytes(b.markers))
        assert np.array_equal(a.get_nodal("lastT"), b.get_nodal("lastT"))


@pytest.mark.parametrize("schedule", ["per_member", "runs", "two_groups"])
@pytest.mark.parametrize("graph", [True, False])
def test_plastic_members_match_members_stepped_alone(graph, schedule):
    """Visco-elasto-plastic members (yielding, so the step's viscosity-only second projection
    and its first projection beside the yield pass on each member's second stream both matter),
    of different sizes, stepped together as captured graphs or on streams: each member's markers
    and nodal fields are what stepping it alone gives, bit for bit"""
    wls = [W.vep_slab_box(nx_cells=nx, ny_cells=ny, nm=4, seed=s)
           for nx, ny, s in ((32, 8, 71), (48, 12, 72), (24, 6, 73))]
    A = [gpu.MicProblem(wl) for wl in wls]
    B = [gpu.MicProblem(wl) for wl in wls]
    E = gpu.MicEnsemble(A)
    E.set_schedule(*SCHEDULES[schedule])
    dts = np.array([wl.dt for wl in wls])
    for _ in range(3):
        E.step(dts, dts, subgrid_stress=1, graph=graph)
        for b, wl in zip(B, wls):
            b.step(wl.dt, wl.dt)
    E.synchronize()
    for a, b in zip(A, B):
        assert np.array_equal(_bytes(a.markers), _bytes(b.markers))
        for f in ("rho", "etaN", "etaS", "soxx", "soxy", "lastT", "kThermal", "dsxx"):
            assert np.array_equal(a.get_nodal(f), b.get_nodal(f)), f


def test_member_stepped_or_tuned_between_replays():
    """A member stepped on its own between captured-graph replays (its step swaps its column
    buffers), or given new launch shapes, must not replay a stale graph: the next ensemble step
    re-captures, and every member still matches the same member stepped alone, bit for bit"""
    wls = _members(60)
    A = _setup(wls)
    B = _setup(wls)
    E = gpu.MicEnsemble(A)
    dts = np.array([wl.dt for wl in wls])

    def both_ensemble():
        E.step(dts, dts, subgrid_stress=1, graph=True)
        for b, dt in zip(B, dts):
            b.step(dt, dt, True)

    for _ in range(3):  # direct step, capture, first replay
        both_ensemble()
    E.synchronize()
    # one member alone: an odd number of buffer swaps relative to the graph's layout
    A[2].step(dts[2], dts[2], True)
    B[2].step(dts[2], dts[2], True)
    for _ in range(3):
        both_ensemble()
    E.synchronize()
    # new launch shapes on one member
    t = A[1].tuning()
    A[1].set_tuning({k: (256 if v != 256 else 128) for k, v in t.items()})
    for _ in range(2):
        both_ensemble()
    E.synchronize()
    for a, b in zip(A, B):
        assert a.n == b.n
        assert np.array_equal(_bytes(a.markers), _bytes(b.markers))
        for f in ("rho", "etaN", "etaS", "lastT"):
            assert np.array_equal(a.get_nodal(f), b.get_nodal(f)), f
    E.close()


@pytest.mark.parametrize("schedule", ["runs", "round_robin", "tile_per_block", "two_groups"])
@pytest.mark.parametrize("graph", [True, False])
def test_creep_members_batched_match_members_stepped_alone(graph, schedule):
    """Law-7 ice members with every yield variant in one batch -- exact creep solve, tensor-core
    surrogate with two different networks, FP32 surrogate -- beside a member without law 7:
    the batched yield kernels restage the network whenever a tile's member uses another one, and
    every member's markers, nodal fields and creep counters are what stepping it alone gives,
    bit for bit"""
    specs = [(24, 24, 0), (32, 16, 2), (16, 40, 2), (40, 24, 1)]
    wls = [W.ice_member(nx, ny, 900 + k) for k, (nx, ny, _) in enumerate(specs)]
    conv = W.convection_member(16, 16, 4, 4, 1e5, 1e2, 77)

    def build():
        out = []
        for wl in wls:
            P = gpu.MicProblem(wl, capacity=wl.capacity)
            gpu.initialize_markers(P, *wl.nm, seed=wl.seed)
            P.set_grain_size(W.ice_grain_sizes(P.n, wl.seed))
            out.append(P)
        P = gpu.MicProblem(conv, capacity=conv.capacity)
        gpu.initialize_markers(P, *conv.nm, seed=conv.seed)
        out.append(P)
        return out

    A, B = build(), build()
    A[1].creep_train(nsamples=1 << 16, batch=1024, steps=300, seed=3)
    net = A[1].creep_params()
    other = net.copy()
    rng = np.random.default_rng(5)
    other[:-16] *= (1.0 + 0.05 * rng.standard_normal(len(other) - 16)).astype(np.float32)
    for k, (_, _, mode) in enumerate(specs):
        for P in (A[k], B[k]):
            P.creep_set_params(other if k == 2 else net)
            P.creep_configure(mode=mode, tol=2e-14, maxit=60, polish_iters=3, polish_tol=1e-7)
    E = gpu.MicEnsemble(A)
    E.set_schedule(*SCHEDULES[schedule])
    dts = np.array([wl.dt for wl in wls] + [conv.dt])
    for _ in range(3):
        E.step(dts, dts, subgrid_stress=1, graph=graph)
        for b, dt in zip(B, dts):
            b.step(dt, dt, True)
        E.synchronize()
        for k in range(len(specs)):
            sa, sb = A[k].creep_stats(), B[k].creep_stats()
            assert sa == sb, (k, sa, sb)
            assert sa["markers"] > 0
    for a, b in zip(A, B):
        assert a.n == b.n
        assert np.array_equal(_bytes(a.markers), _bytes(b.markers))
        for f in ("rho", "etaN", "etaS", "soxx", "lastT"):
            assert np.array_equal(a.get_nodal(f), b.get_nodal(f)), f
    E.close()
