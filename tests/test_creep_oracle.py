"""CPU checks of the composite-creep oracle: the exact stress solve on the reference law, and
the FP64 surrogate network gradient against finite differences."""
import numpy as np

from fvmic2d_gb300 import workloads as W
from oracle import mlp_oracle as M
from oracle import oraclepy


def creep_samples(n, seed):
    u = W.splitmix64_uniform(seed, 4 * n)
    edot = 10 ** (-18 + 8 * u[0::4])
    T = 100 + 173 * u[1::4]
    d = 10 ** (-4 + 3 * u[2::4])
    P = 1e8 * u[3::4]
    return edot, T, d, P


def test_oracle_creep_stress_meets_reference_law():
    edot, T, d, P = creep_samples(3000, 11)
    # parameter switches of the law (viscosity.c:138, 154), tiny and large rates, P below 1 Pa
    edot = np.concatenate([edot, [1e-18, 1e-10, 3e-14, 3e-14, 3e-14, 3e-14, 1e-12]])
    T = np.concatenate([T, [100.0, 273.0, 254.999, 255.0, 257.999, 258.0, 200.0]])
    d = np.concatenate([d, [1e-4, 1e-1, 1e-3, 1e-3, 1e-3, 1e-3, 1e-2]])
    P = np.concatenate([P, [0.0, 1e8, 5e7, 5e7, 5e7, 5e7, 0.3]])
    s, it = oraclepy.creep_stress(edot, T, d, P)
    rate = oraclepy.gk_strain_rate(s, T, d, P)
    rel = np.abs(rate / edot - 1.0)
    jump = s == 1.0  # the law's rate jumps at s = 1 Pa: a root inside the jump is reported as 1 Pa
    assert np.all(rel[~jump] <= 1e-13), rel[~jump].max()
    assert np.all(it < 100)


def test_surrogate_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = np.zeros(M.N_PARAMS)
    p[:M.N_TRAIN] = rng.normal(0, 0.3, M.N_TRAIN)
    p[M.OFF_NORM], p[M.OFF_NORM + 1] = 5.0, 1.5
    X = rng.uniform(-1, 1, (64, 4))
    t = rng.normal(5.0, 1.5, 64)
    loss, g = M.loss_and_grad(p, X, t)
    idx = rng.choice(M.N_TRAIN, 60, replace=False)
    for k in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_only(pp, X, t) - M.loss_only(pm, X, t)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, fd, g[k])
