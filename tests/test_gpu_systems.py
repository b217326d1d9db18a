"""GPU assembly of the two linear systems of a time step against the reference's own outputs
(formVEPSystem, enforceThermalBCs1, formThermalSystem; golden vectors), and the device's direct
solve against a host sparse LU of the same matrices."""
import os

import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from tests.helpers import exact
from tests.test_oracle_pin import SYSTEM_KINDS, systems_case_from_golden

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    return np.load(os.path.join(GOLDEN, "linear_systems.npz"))


def _csr(z, kind, name):
    return tuple(z["%s_%s_%s" % (kind, name, k)] for k in ("rowptr", "cols", "vals", "rhs"))


def _problem(z, kind, build="product"):
    wl, so, dt = systems_case_from_golden(z, kind)
    return gpu.MicProblem(wl, exact=(build == "exact")), so, dt


def _same_system(got, ref, name):
    for k, a, b in zip(("rowptr", "cols", "vals", "rhs"), got, ref):
        if k in ("rowptr", "cols"):
            assert np.array_equal(a, b), (name, k)
        else:
            ok, msg = exact(a, b)
            assert ok, (name, k, msg)


@pytest.mark.parametrize("build", ["exact", "product"])
@pytest.mark.parametrize("kind", list(SYSTEM_KINDS))
def test_assembly_matches_reference_outputs(kind, build):
    """every entry, column and right-hand side value bit-identical to the reference's"""
    z = _golden()
    G, so, dt = _problem(z, kind, build)
    kb, kc = G.formVEPSystem(so, dt)
    assert (kb, kc) == tuple(z[kind + "_K"])
    _same_system(G.system(G.STOKES), _csr(z, kind, "stokes"), "stokes")
    G.enforceThermalBCs1(so)
    ok, msg = exact(G.get_nodal("lastT"), z[kind + "_lastT"])
    assert ok, msg
    G.formThermalSystem(so, dt)
    _same_system(G.system(G.THERMAL), _csr(z, kind, "thermal"), "thermal")


def _spsolve(rp, c, v, rhs):
    sp = pytest.importorskip("scipy.sparse")
    spl = pytest.importorskip("scipy.sparse.linalg")
    n = len(rp) - 1
    A = sp.csr_matrix((v, c, rp), shape=(n, n))
    return A, spl.spsolve(A.tocsc(), rhs)


@pytest.mark.parametrize("kind", list(SYSTEM_KINDS))
def test_direct_solve_matches_host_lu(kind):
    """the device's banded LU against a host sparse LU (SuperLU) of the same matrix: solutions
    within 1e-9 relative for Stokes (condition numbers near 1e8 with four decades of viscosity)
    and 1e-12 for temperature, residuals at rounding level"""
    z = _golden()
    G, so, dt = _problem(z, kind)
    G.formVEPSystem(so, dt)
    G.linear_solve(G.STOKES)
    x = G.solution(G.STOKES)
    A, xr = _spsolve(*_csr(z, kind, "stokes"))
    b = z["%s_stokes_rhs" % kind]
    assert np.all(np.isfinite(x))
    assert np.max(np.abs(x - xr)) <= 1e-9 * np.max(np.abs(xr))
    assert np.max(np.abs(A @ x - b)) <= 1e-12 * np.max(np.abs(A).sum(axis=1)) * np.max(np.abs(x))
    kl, ku = G.system_band(G.STOKES)
    assert 0 < kl <= 3 * (min(G.NX, G.NY) + 2) and 0 < ku <= 3 * (min(G.NX, G.NY) + 2)
    G.enforceThermalBCs1(so)
    G.formThermalSystem(so, dt)
    G.linear_solve(G.THERMAL)
    T = G.solution(G.THERMAL)
    A, Tr = _spsolve(*_csr(z, kind, "thermal"))
    assert np.max(np.abs(T - Tr)) <= 1e-12 * np.max(np.abs(Tr))
    assert np.array_equal(G.get_nodal("thisT").ravel(), T)


def test_solution_feeds_retrieve_solutions():
    """retrieveSolutions from the device-resident solution gives what it gives from the same
    vector passed from the host"""
    z = _golden()
    G, so, dt = _problem(z, "fixed_top")
    kb, kc = G.formVEPSystem(so, dt)
    G.linear_solve(G.STOKES)
    x = G.solution(G.STOKES)
    G.retrieveSolutions(None, kc)
    dev = {f: G.get_nodal(f) for f in ("vx", "vy", "p")}
    G.retrieveSolutions(x, kc)
    for f in ("vx", "vy", "p"):
        assert np.array_equal(dev[f], G.get_nodal(f)), f


def test_solve_larger_grid_residual():
    """a 129 x 33 node box (37,539 Stokes unknowns, band about 100 on each side): the solve's
    residual stays at rounding level"""
    from tests.test_oracle_pin import systems_case
    from fvmic2d_gb300 import workloads as W

    wl, so, dt = systems_case("fixed_top")
    big = W.vep_slab_box(nx_cells=128, ny_cells=32, nm=2, seed=3)
    g = big.grid
    u = W.splitmix64_uniform(41, 8 * g.NX * g.NY).reshape(8, g.NY, g.NX)
    big.nodal.update({"etaN": 10 ** (19 + 3 * u[0]), "etaS": 10 ** (19 + 3 * u[1]), "muN": 1e10 * (0.5 + u[2]),
                      "muS": 1e10 * (0.5 + u[3]), "rho": 30 * (u[4] - 0.5), "rhodot": 0 * u[5]})
    so.overridingPlateThickness = 0.3 * g.LY
    so.slabAngle = 0.8
    so.rootCenter = 0.5 * g.LX
    so.rootWidth = 0.2 * g.LX
    so.rootThickness = 0.05 * g.LY
    G = gpu.MicProblem(big)
    G.formVEPSystem(so, dt)
    G.linear_solve(G.STOKES)
    x = G.solution(G.STOKES)
    rp, c, v, rhs = G.system(G.STOKES)
    sp = pytest.importorskip("scipy.sparse")
    A = sp.csr_matrix((v, c, rp), shape=(len(rhs), len(rhs)))
    assert np.all(np.isfinite(x))
    assert np.max(np.abs(A @ x - rhs)) <= 1e-11 * np.max(np.abs(A).sum(axis=1)) * np.max(np.abs(x))


def test_repeated_solves_replay_the_same_factorisation():
    """The first solve of a system captures its factorisation as a CUDA graph; later solves of the
    same shape replay it.  Stokes and thermal solves alternate over one shared factorisation
    buffer: every replay gives the first solve's answer bit for bit, and the launch counter counts
    the replayed kernels."""
    z = _golden()
    G, so, dt = _problem(z, "fixed_top")
    G.formVEPSystem(so, dt)
    G.enforceThermalBCs1(so)
    G.formThermalSystem(so, dt)
    first = {}
    launches = []
    for rnd in range(3):
        for which in (G.STOKES, G.THERMAL):
            l0 = G.launch_count()
            G.linear_solve(which)
            launches.append((which, G.launch_count() - l0))
            x = G.solution(which)
            if rnd == 0:
                first[which] = x
            else:
                assert np.array_equal(x, first[which]), (rnd, which)
    for which in (G.STOKES, G.THERMAL):
        counts = [c for w, c in launches if w == which]
        assert counts[0] > 10 and len(set(counts)) == 1, counts
