"""GPU checks of device paths that the step tests reach only indirectly: the division by a
grid spacing that decides the 0.5-tie tests of the projection and sub-grid passes, and
projectNodalFieldToMarkersS (markers.c:1670-1706) called on its own."""
import numpy as np
import pytest

from fvmic2d_gb300 import gpu, workloads as W
from oracle import oraclepy
from tests.helpers import compare_markers

pytestmark = pytest.mark.gpu


def _bits_to_f64(b):
    return np.asarray(b, dtype=np.uint64).view(np.float64)


def _division_cases():
    rng = np.random.default_rng(2024)
    n = 1 << 18
    # grid spacings over many binades and offsets inside the spacing (quotients in [0, 1))
    den = 10.0 ** rng.uniform(-4, 6, n)
    num = den * rng.uniform(0, 1, n)
    cases = [(num, den)]
    # divisors with an all-ones mantissa (their reciprocal is just above a power of two) and
    # with a mantissa of one plus one ulp, at several exponents
    e = rng.integers(1000, 1046, 4096).astype(np.uint64)
    ones = _bits_to_f64((e << np.uint64(52)) | np.uint64((1 << 52) - 1))
    one_ulp = _bits_to_f64((e << np.uint64(52)) | np.uint64(1))
    for d in (ones, one_ulp):
        cases.append((d * rng.uniform(0, 1, len(d)), d))
    # quotients at exactly 0.5, 0.25, 0.75, and a few ulps either side of 0.5
    d = 10.0 ** rng.uniform(-3, 5, 8192)
    for q in (0.5, 0.25, 0.75):
        cases.append((d * q, d))
    half = d * 0.5
    for k in (1, 2, 3):
        cases.append((np.nextafter(half, np.inf) if k == 1 else half + k * np.spacing(half), d))
        cases.append((np.nextafter(half, 0.0) if k == 1 else half - k * np.spacing(half), d))
    # numerators whose exact quotient lies next to a rounding boundary: num = RN(q * den) for
    # representable q, and the midpoints between consecutive quotients
    q = rng.uniform(0, 1, n)
    d = 10.0 ** rng.uniform(-3, 5, n)
    cases.append((q * d, d))
    cases.append(((q + np.spacing(q) / 2) * d, d))
    num = np.concatenate([c[0] for c in cases])
    den = np.concatenate([c[1] for c in cases])
    return num, den


@pytest.mark.parametrize("exact_build", [False, True])
def test_grid_spacing_division_is_correctly_rounded(exact_build):
    """div_sp (reciprocal multiply plus one residual correction, Markstein's theorem) returns the
    correctly rounded quotient, bit for bit equal to IEEE division, over random and adversarial
    divisors and quotients at and around the 0.5 ties"""
    G = gpu.MicProblem(W.convection_box(ncell=4, nm=2, seed=1), exact=exact_build)
    num, den = _division_cases()
    got = G.debug_div_sp(num, den)
    want = num / den
    bad = got.view(np.uint64) != want.view(np.uint64)
    assert not bad.any(), (int(bad.sum()), num[bad][:4], den[bad][:4], got[bad][:4], want[bad][:4])
    G.close()


@pytest.mark.parametrize("exact_build", [False, True])
@pytest.mark.parametrize("case", ["convection", "vep_refined"])
def test_project_nodal_field_to_markers_matches_oracle(exact_build, case):
    """projectNodalFieldToMarkersS of a basic-node field onto a marker field, on its own (the
    initial temperature of main_subduction.c:202): within 1e-12 of the oracle in the product
    build, bit for bit in the FMA-free build; markers outside the domain keep their value"""
    wl = (W.convection_box(ncell=24, nm=4, seed=8) if case == "convection"
          else W.vep_slab_box(nx_cells=48, ny_cells=12, nm=3, seed=9))
    rng = np.random.default_rng(5)
    field = rng.uniform(-1.0, 2.0, (wl.grid.NY, wl.grid.NX))
    m = wl.markers.copy()
    m["X"][:7] = [-1.0, wl.grid.LX * 1.5, 0.0, wl.grid.LX, 0.5 * wl.grid.LX, np.nan, wl.grid.x[3]]
    m["Y"][:7] = [0.3 * wl.grid.LY, 0.2 * wl.grid.LY, 0.0, wl.grid.LY, -2.0, 0.5, wl.grid.y[2]]
    G = gpu.MicProblem(wl, markers=m, exact=exact_build)
    O = oraclepy.OracleProblem(wl, markers=m)
    for P in (G, O):
        P.set_nodal("thisT", field)
        P.findMarkerCells()
        P.projectNodalFieldToMarkersS("thisT", "T")
    fails = compare_markers(G.markers, O.markers, rtol=None if exact_build else 1e-12)
    assert not fails, fails
    assert np.array_equal(G.markers["T"][[0, 1, 4]], m["T"][[0, 1, 4]])
    G.close()
