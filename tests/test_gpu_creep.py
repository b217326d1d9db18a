"""GPU checks of the composite ice creep closure (law 7): exact solve, training gradients,
the trained surrogate with FP64 polish and exact fallback, and law 7 inside the marker pass."""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from oracle import mlp_oracle as M
from oracle import oraclepy
from tests.helpers import close
from tests.test_creep_oracle import creep_samples

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    wl = W.ice_creep_box(nx_cells=16, ny_cells=16, nm=2, seed=4)
    G = gpu.MicProblem(wl)
    G.set_grain_size(wl.grain_size)
    return G, wl


def test_exact_solve_matches_oracle_and_reference_law(ctx):
    G, _ = ctx
    edot, T, d, P = creep_samples(20000, 21)
    edot = np.concatenate([edot, [1e-18, 1e-10, 3e-14, 3e-14, 3e-14, 3e-14, 1e-12, 0.0]])
    T = np.concatenate([T, [100.0, 273.0, 254.999, 255.0, 257.999, 258.0, 200.0, 200.0]])
    d = np.concatenate([d, [1e-4, 1e-1, 1e-3, 1e-3, 1e-3, 1e-3, 1e-2, 1e-3]])
    P = np.concatenate([P, [0.0, 1e8, 5e7, 5e7, 5e7, 5e7, 0.3, 1e5]])
    s, it, res, _ = G.creep_solve(edot, T, d, P, mode=0)
    sub = slice(0, None, 7)  # the oracle solve is a Python loop: check every 7th sample
    s_o, _ = oraclepy.creep_stress(edot[sub], T[sub], d[sub], P[sub])
    ok, msg = close(s[sub], s_o, 1e-12)
    assert ok, msg
    pos = edot > 0
    rate = oraclepy.gk_strain_rate(s[pos][::3], T[pos][::3], d[pos][::3], P[pos][::3])
    rel = np.abs(rate / edot[pos][::3] - 1.0)
    jump = s[pos][::3] == 1.0
    assert np.all(rel[~jump] <= 1e-13), rel[~jump].max()
    assert it.max() < 60 and s[-1] == 0.0


def test_training_gradient_matches_fp64_oracle(ctx):
    G, _ = ctx
    rng = np.random.default_rng(9)
    p = np.zeros(M.N_PARAMS, dtype=np.float32)
    p[:M.N_TRAIN] = rng.normal(0, 0.3, M.N_TRAIN)
    p[M.OFF_NORM], p[M.OFF_NORM + 1] = 5.0, 1.5
    X = rng.uniform(-1, 1, (512, 4)).astype(np.float32)
    t = rng.normal(5.0, 1.5, 512).astype(np.float32)
    g, loss = G.creep_grad(p, X, t)
    # quantization-aware: the library's forward and backward use W2 rounded to BF16
    loss_o, g_o = M.loss_and_grad(p.astype(np.float64), X.astype(np.float64), t.astype(np.float64), w2_bf16=True)
    assert abs(loss - loss_o) <= 1e-4 * loss_o
    assert np.linalg.norm(g - g_o) <= 1e-4 * np.linalg.norm(g_o)
    # every parameter block individually
    for a, b in [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.OFF_NORM)]:
        assert np.linalg.norm(g[a:b] - g_o[a:b]) <= 2e-4 * np.linalg.norm(g_o[a:b]) + 1e-7


def _random_params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.N_PARAMS, dtype=np.float32)
    p[M.OFF_W1:M.OFF_B1] = rng.uniform(-1.2, 1.2, M.OFF_B1 - M.OFF_W1)
    p[M.OFF_B1:M.OFF_W2] = rng.uniform(-0.5, 0.5, M.H)
    p[M.OFF_W2:M.OFF_B2] = rng.uniform(-0.3, 0.3, M.H * M.H)
    p[M.OFF_B2:M.OFF_W3] = rng.uniform(-0.5, 0.5, M.H)
    p[M.OFF_W3:M.OFF_B3] = rng.uniform(-0.3, 0.3, M.H)
    p[M.OFF_B3], p[M.OFF_NORM], p[M.OFF_NORM + 1] = 0.1, 5.0, 1.5
    return p


@pytest.mark.parametrize("n", [1, 127, 1000, 128 * 4 * 152 * 2 + 7])
def test_tensor_core_network_matches_fp64_forward(ctx, n):
    """The tcgen05 path (BF16 W2, activations as two BF16 pieces, FP32 accumulation in tensor
    memory) against the FP64 NumPy forward pass of the same network (W2 rounded to BF16, as the
    library holds it) and the FP32 CUDA-core path; ragged tile counts and more tiles than
    persistent blocks."""
    G, _ = ctx
    p = _random_params(n)
    G.creep_set_params(p)
    X = np.random.default_rng(n + 1).uniform(-1, 1, (n, 4)).astype(np.float32)
    y64, (_, h1, z2, h2) = M.forward(p.astype(np.float64), X.astype(np.float64), w2_bf16=True)
    # error scale: magnitude of the terms summed in the hidden and output layers
    scale = 1.0 + np.abs(h2) @ np.abs(p[M.OFF_W3:M.OFF_B3].astype(np.float64))
    y1 = G.creep_infer(X, mode=1)
    y2 = G.creep_infer(X, mode=2)
    assert G.creep_stats()["tc_timeouts"] == 0
    assert np.all(np.abs(y1 - y64) <= 2e-6 * scale), np.abs(y1 - y64).max()
    assert np.all(np.abs(y2 - y64) <= 2e-5 * scale), np.abs(y2 - y64).max()


@pytest.fixture(scope="module")
def trained(ctx):
    G, _ = ctx
    hist = G.creep_train(nsamples=1 << 21, batch=4096, steps=10000, lr=3e-3, seed=1)
    return G, hist


def test_training_converges(trained):
    _, hist = trained
    assert hist[-50:].mean() < 0.02 * hist[:50].mean()


def test_surrogate_polish_meets_tolerance_and_saves_iterations(trained):
    """What the trained network gains: stresses within 1e-6 of the exact solve (the polish
    tolerance 1e-7 on the rate residual) from under 60% of its FP64 Newton iterations, with
    almost no exact fallbacks, on both inference paths."""
    G, _ = trained
    edot, T, d, P = creep_samples(200000, 77)
    G.creep_configure(mode=0, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    s_exact, it_exact, _, _ = G.creep_solve(edot, T, d, P, mode=0)
    for mode in (1, 2):
        s_sur, it_sur, res, fb = G.creep_solve(edot, T, d, P, mode=mode)
        rel = np.abs(s_sur / s_exact - 1.0)
        assert rel.max() <= 1e-6, (mode, rel.max())
        assert fb.mean() < 0.01, (mode, fb.mean())
        assert it_sur.mean() < 0.6 * it_exact.mean(), (mode, it_sur.mean(), it_exact.mean())
        assert np.all(np.abs(res) <= 1e-7)


def test_surrogate_modes_converge_to_the_exact_root(trained):
    """With the polish tolerance at the exact tolerance, both surrogate paths return the exact
    solve's stress (<= 1e-12 relative) from fewer FP64 Newton iterations."""
    G, _ = trained
    edot, T, d, P = creep_samples(300001, 78)
    G.creep_configure(mode=0, tol=2e-14, polish_iters=6, polish_tol=2e-14)
    s0, it0, _, _ = G.creep_solve(edot, T, d, P, mode=0)
    for mode in (1, 2):
        s, it, res, fb = G.creep_solve(edot, T, d, P, mode=mode)
        ok, msg = close(s, s0, 1e-12)
        assert ok, (mode, msg)
        st = G.creep_stats()
        assert st["tc_timeouts"] == 0 and st["max_residual"] <= 2e-14
        assert fb.mean() < 0.01, (mode, fb.mean())
        assert it.mean() < 0.8 * it0.mean(), (mode, it.mean(), it0.mean())


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_law7_marker_pass_matches_oracle(trained, mode):
    wl = W.ice_creep_box(nx_cells=24, ny_cells=24, nm=3, seed=5)
    G = gpu.MicProblem(wl)
    G.set_grain_size(wl.grain_size)
    if mode:
        G.creep_set_params(trained[0].creep_params())
    G.creep_configure(mode=mode, tol=2e-14, polish_iters=6, polish_tol=2e-14)
    O = oraclepy.OracleProblem(wl)
    O.set_grain_size(wl.grain_size)
    G.findMarkerCells()
    O.findMarkerCells()
    G.checkPlasticYielding(wl.dt)
    O.checkPlasticYielding(wl.dt)
    ok, msg = close(G.markers["eta"], O.markers["eta"], 1e-12)
    assert ok, msg
    st = G.creep_stats()
    assert st["markers"] == len(wl.markers) and st["tc_timeouts"] == 0
    assert st["fallbacks"] <= 0.01 * len(wl.markers)
    assert st["max_residual"] <= 2e-14


def test_tensor_core_wait_that_runs_out_falls_back_to_exact(trained):
    """The bounded wait on each tensor-core tile's completion, made to run out (a limit of zero
    try_wait rounds): every block gives up on its first tile and counts it, drains the committed
    MMA before freeing its tensor memory, and every non-linear marker takes the exact solve --
    stresses bit for bit those of mode 0.  The context stays usable: with the default limit the
    next solve uses the tensor cores again."""
    G, _ = trained
    edot, T, d, P = creep_samples(100000, 79)
    G.creep_configure(mode=0, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    s0, _, _, _ = G.creep_solve(edot, T, d, P, mode=0)
    G.creep_set_tc_wait_limit(0)
    try:
        s, _, res, fb = G.creep_solve(edot, T, d, P, mode=2)
        st, tcs = G.creep_stats(), G.creep_tc_stats()
    finally:
        G.creep_set_tc_wait_limit(1 << 20)
    assert st["tc_timeouts"] > 0 and tcs["tile_timeouts"] == st["tc_timeouts"]
    assert tcs["drain_timeouts"] == 0
    # the non-linear branch (s* >= 1 Pa) is where the network would have been used
    nonlinear = (edot > 0) & (s0 >= 1.0)
    assert nonlinear.any() and np.array_equal(fb == 1, nonlinear)
    assert st["fallbacks"] == int(fb.sum())
    assert np.array_equal(s.view(np.uint64), s0.view(np.uint64))
    s2, _, _, fb2 = G.creep_solve(edot, T, d, P, mode=2)
    assert G.creep_tc_stats() == {"tile_timeouts": 0, "drain_timeouts": 0}
    assert fb2.mean() < 0.01
    assert np.max(np.abs(s2 / s0 - 1.0)) <= 1e-6


def test_tensor_core_wait_that_runs_out_in_the_marker_pass(trained):
    """The same give-up inside checkPlasticYielding's tensor-core pass: viscosities bit for bit
    those of the exact pass, tiles counted, and the context usable afterwards"""
    wl = W.ice_creep_box(nx_cells=24, ny_cells=24, nm=3, seed=6)
    A = gpu.MicProblem(wl)
    B = gpu.MicProblem(wl)
    for G in (A, B):
        G.set_grain_size(wl.grain_size)
        G.findMarkerCells()
    B.creep_set_params(trained[0].creep_params())
    A.creep_configure(mode=0, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    B.creep_configure(mode=2, tol=2e-14, polish_iters=3, polish_tol=1e-7)
    B.creep_set_tc_wait_limit(0)
    A.checkPlasticYielding(wl.dt)
    B.checkPlasticYielding(wl.dt)
    tcs = B.creep_tc_stats()
    assert tcs["tile_timeouts"] > 0 and tcs["drain_timeouts"] == 0
    assert np.array_equal(A.markers["eta"].view(np.uint64), B.markers["eta"].view(np.uint64))
    B.creep_set_tc_wait_limit(1 << 20)
    B.checkPlasticYielding(wl.dt)
    assert B.creep_tc_stats()["tile_timeouts"] == 0
    A.close()
    B.close()
