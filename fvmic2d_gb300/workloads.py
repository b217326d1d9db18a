"""Seeded synthetic workloads for the marker-in-cell transfer path.

No public dataset exists for this path; every input is generated here from a
SplitMix64 stream so that the CPU oracle, the reference build and the GPU see
identical arrays.  Marker placement follows fvmic2d's
``distributeMarkersUniformInDomain`` (markers.c:342-400): a domain-uniform
lattice of NMX*(NX-1) by NMY*(NY-1) markers, each jittered by U(-d/4, d/4) per
axis, stored x-major (lattice column outer, row inner), so the initial array is
not in cell order.  Cell centres follow ``getCellCenters`` (gridSpacing.c:150-157).

Nodal inputs that the host Stokes / thermal solves would produce (vx, vy, p,
strain rates, vorticity, nodal stresses and stress changes, the new
temperature) are sampled from a prescribed divergence-free velocity field.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from .mic_types import MARKER_DTYPE, Materials, Options, BCs

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_uniform(seed, n, offset=0):
    """n uniforms in [0,1) from SplitMix64 (Steele, Lea & Flood 2014), stream position offset.."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def spacing_uniform(xmin, xmax, n):
    """gridSpacingUniform (gridSpacing.c:8-17): running sum of a constant step."""
    x = np.empty(n)
    dx = (xmax - xmin) / (n - 1.0)
    x[0] = xmin
    acc = xmin
    for i in range(1, n - 1):
        acc = acc + dx
        x[i] = acc
    x[n - 1] = xmax
    return x


def cell_centers(x, L):
    n = len(x)
    xc = np.empty(n + 1)
    xc[1:n] = (x[:-1] + x[1:]) / 2.0
    xc[0] = -xc[1]
    xc[n] = 2.0 * L - xc[n - 1]
    return xc


@dataclass
class Grid:
    NX: int
    NY: int
    LX: float
    LY: float
    x: np.ndarray
    y: np.ndarray

    def __post_init__(self):
        self.x = np.ascontiguousarray(self.x, dtype=np.float64)
        self.y = np.ascontiguousarray(self.y, dtype=np.float64)
        self.xc = cell_centers(self.x, self.LX)
        self.yc = cell_centers(self.y, self.LY)

    @property
    def ncells(self):
        return (self.NX - 1) * (self.NY - 1)


@dataclass
class Workload:
    name: str
    grid: Grid
    markers: np.ndarray
    materials: Materials
    options: Options
    bcs: BCs
    nodal: dict = field(default_factory=dict)
    dt: float = 0.0            # displacement time step (stress update, subgrid stress)
    dt_thermal: float = 0.0    # thermal time step (subgrid temperature, advection)
    steps: int = 1
    grain_size: np.ndarray = None  # per-marker grain size (composite creep workloads)


def lattice_markers(grid, nmx, nmy, seed):
    """Domain-uniform jittered lattice in x-major order (markers.c:369-395)."""
    mdx = grid.LX / (nmx * (grid.NX - 1))
    mdy = grid.LY / (nmy * (grid.NY - 1))
    nk = int((grid.x[-1] - grid.x[0]) / mdx + 1e-9)
    nl = int((grid.y[-1] - grid.y[0]) / mdy + 1e-9)
    n = nk * nl
    u = splitmix64_uniform(seed, 2 * n)
    k = np.repeat(np.arange(nk, dtype=np.float64), nl)
    l = np.tile(np.arange(nl, dtype=np.float64), nk)
    m = np.zeros(n, dtype=MARKER_DTYPE)
    m["X"] = grid.x[0] + mdx * (0.5 + k) + (-mdx / 4.0 + (mdx / 2.0) * u[0::2])
    m["Y"] = grid.y[0] + mdy * (0.5 + l) + (-mdy / 4.0 + (mdy / 2.0) * u[1::2])
    m["Mat"] = 0
    m["cellX"] = -1
    m["cellY"] = -1
    return m


def _materials(n):
    mat = Materials()
    mat.nMaterials = n
    return mat


def _free_slip():
    b = BCs()
    for side in (b.mechBCLeft, b.mechBCRight, b.mechBCTop, b.mechBCBottom):
        for c in range(3):
            side.type[c] = 1
            side.value[c] = 0.0
    return b


def _eta_law(mat, m):
    """computeRheology (viscosity.c:12-67) for hasEtaT in {0, 1, 5}, vectorised; clamp done by caller."""
    eta = np.empty(len(m))
    for k in range(mat.nMaterials):
        sel = m["Mat"] == k
        law = mat.hasEtaT[k]
        if law == 0:
            eta[sel] = mat.materialEta[k]
        elif law == 1:
            eta[sel] = mat.materialEta[k] * np.exp(mat.QonR[k] * (1.0 / m["T"][sel] - 1.0 / mat.Tref[k]))
        elif law == 5:
            eta[sel] = mat.materialEta[k] * np.exp(-mat.QonR[k] * m["T"][sel])
        else:
            raise ValueError("unsupported law in generator")
    return eta


def _velocity_fields(grid, vx_fn, vy_fn, dvx, dvy):
    """Sample vx at (x[i], yc[j+1]), vy at (xc[i+1], y[j]) (markers.c:1978-1984, 2026-2029),
    strain rates / vorticity at cell centres (xx, yy) and basic nodes (xy, wxy)."""
    X, YC = np.meshgrid(grid.x, grid.yc[1:], indexing="xy")
    XC, Y = np.meshgrid(grid.xc[1:], grid.y, indexing="xy")
    vx = vx_fn(X, YC)
    vy = vy_fn(XC, Y)
    XCc, YCc = np.meshgrid(grid.xc[: grid.NX], grid.yc[: grid.NY], indexing="xy")
    Xb, Yb = np.meshgrid(grid.x, grid.y, indexing="xy")
    exx = dvx["x"](XCc, YCc)
    eyy = dvy["y"](XCc, YCc)
    exy = 0.5 * (dvx["y"](Xb, Yb) + dvy["x"](Xb, Yb))
    wxy = 0.5 * (dvx["y"](Xb, Yb) - dvy["x"](Xb, Yb))
    return vx, vy, exx, eyy, exy, wxy


def convection_box(ncell=64, nm=4, seed=1, U=100.0):
    """Unit-square thermal convection, viscosity exp(-ln(1000) T) (hasEtaT 5), free slip,
    T0 = 1 - y + 0.01 cos(pi x) sin(pi y); 65x65 nodes and 65,536 markers at full size."""
    NX = NY = ncell + 1
    g = Grid(NX, NY, 1.0, 1.0, spacing_uniform(0.0, 1.0, NX), spacing_uniform(0.0, 1.0, NY))
    m = lattice_markers(g, nm, nm, seed)
    m["T"] = 1.0 - m["Y"] + 0.01 * np.cos(np.pi * m["X"]) * np.sin(np.pi * m["Y"])
    mat = _materials(1)
    mat.materialEta[0] = 1.0
    mat.materialRho[0] = 1.0
    mat.materialkThermal[0] = 1.0
    mat.materialCp[0] = 1.0
    mat.materialAlpha[0] = 1.0
    mat.materialMu[0] = 1e20
    mat.hasEtaT[0] = 5
    mat.QonR[0] = math.log(1000.0)
    mat.Tref[0] = 1.0
    opt = Options(etamin=1e-3, etamax=1e3, fractionalEtamin=0.01, subgridStressDiffusivity=0.0,
                  subgridTemperatureDiffusivity=1.0)
    m["mu"] = mat.materialMu[0]
    m["eta"] = _eta_law(mat, m)
    pi = np.pi
    vx_fn = lambda x, y: U * pi * np.sin(pi * x) * np.cos(pi * y)
    vy_fn = lambda x, y: -U * pi * np.cos(pi * x) * np.sin(pi * y)
    dvx = {"x": lambda x, y: U * pi * pi * np.cos(pi * x) * np.cos(pi * y),
           "y": lambda x, y: -U * pi * pi * np.sin(pi * x) * np.sin(pi * y)}
    dvy = {"x": lambda x, y: U * pi * pi * np.sin(pi * x) * np.sin(pi * y),
           "y": lambda x, y: -U * pi * pi * np.cos(pi * x) * np.cos(pi * y)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    ex_m = dvx["x"](m["X"], m["Y"])
    m["exx"] = ex_m
    m["eyy"] = -ex_m
    m["exy"] = 0.0
    m["sxx"] = 2.0 * m["eta"] * m["exx"]
    m["syy"] = -m["sxx"]
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    Tn = 1.0 - Yb + 0.01 * np.cos(pi * Xb) * np.sin(pi * Yb)
    eta_c = np.exp(-math.log(1000.0) * np.clip(1.0 - YCc, 0.0, 1.0))
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": np.zeros((NY, NX)),
        "soxx": 2.0 * eta_c * exx, "soyy": 2.0 * eta_c * eyy, "soxy": np.zeros((NY, NX)),
        "thisT": Tn + 1e-3 * np.sin(pi * Xb) * np.sin(pi * Yb),
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * exy
    dt = 0.5 * (1.0 / ncell) / (U * pi)
    return Workload("convection_box", g, m, mat, opt, _free_slip(), nodal, dt, dt, 10)


def refined_top_y(LY, ny_cells, top_fraction=0.2):
    """y gridlines with the top `top_fraction` of the box at about twice the resolution."""
    n_top = max(1, min(ny_cells - 1, int(round(ny_cells * 2.0 * top_fraction / (1.0 + top_fraction)))))
    n_bot = ny_cells - n_top
    y_top = spacing_uniform(0.0, top_fraction * LY, n_top + 1)
    y_bot = spacing_uniform(top_fraction * LY, LY, n_bot + 1)
    return np.concatenate([y_top, y_bot[1:]])


def vep_slab_box(nx_cells=1024, ny_cells=256, nm=4, seed=2):
    """Visco-elasto-plastic two-material 4:1 box: dense slab rectangle (material 1, Mohr-Coulomb
    yield C + F p) in a lighter Arrhenius mantle (material 0); eta clamped to [1e19, 1e23] Pa s,
    shear modulus 1e10 Pa; y spacing about 2x finer in the top 20 %.  At full size
    1025 x 257 nodes and 4,194,304 markers."""
    NX, NY = nx_cells + 1, ny_cells + 1
    LX, LY = 4.0e5, 1.0e5
    g = Grid(NX, NY, LX, LY, spacing_uniform(0.0, LX, NX), refined_top_y(LY, ny_cells))
    m = lattice_markers(g, nm, nm, seed)
    u = splitmix64_uniform(seed + 1000, len(m))
    X, Y = m["X"], m["Y"]
    slab = (X > 0.35 * LX) & (X < 0.65 * LX) & (Y > 0.05 * LY) & (Y < 0.35 * LY)
    m["Mat"] = np.where(slab, 1, 0)
    Tgeo = 273.0 + 1300.0 * np.minimum(1.0, Y / (0.4 * LY))
    m["T"] = np.where(slab, 273.0 + 0.5 * (Tgeo - 273.0), Tgeo) + 5.0 * (u - 0.5)
    mat = _materials(2)
    for k, (eta, rho) in enumerate([(1e21, 3300.0), (1e23, 3400.0)]):
        mat.materialEta[k] = eta
        mat.materialRho[k] = rho
        mat.materialkThermal[k] = 3.0
        mat.materialCp[k] = 1250.0
        mat.materialAlpha[k] = 3e-5
        mat.materialMu[k] = 1e10
        mat.Tref[k] = 1573.0
    mat.hasEtaT[0] = 1
    mat.QonR[0] = 2.0e4
    mat.hasEtaT[1] = 0
    mat.hasPlasticity[1] = 1
    mat.materialCohesion[1] = 2e7
    mat.materialFriction[1] = 0.6
    opt = Options(etamin=1e19, etamax=1e23, fractionalEtamin=0.1, subgridStressDiffusivity=1.0,
                  subgridTemperatureDiffusivity=1.0)
    edot, gdot = 1e-15, 4e-16
    A = 0.3 * edot * LX * LY / np.pi
    pi = np.pi
    vx_fn = lambda x, y: edot * (x - LX / 2) + gdot * (y - LY / 2) + A * pi / LY * np.sin(pi * x / LX) * np.cos(pi * y / LY)
    vy_fn = lambda x, y: -edot * (y - LY / 2) - A * pi / LX * np.cos(pi * x / LX) * np.sin(pi * y / LY)
    dvx = {"x": lambda x, y: edot + A * pi * pi / (LX * LY) * np.cos(pi * x / LX) * np.cos(pi * y / LY),
           "y": lambda x, y: gdot - A * pi * pi / (LY * LY) * np.sin(pi * x / LX) * np.sin(pi * y / LY)}
    dvy = {"x": lambda x, y: A * pi * pi / (LX * LX) * np.sin(pi * x / LX) * np.sin(pi * y / LY),
           "y": lambda x, y: -edot - A * pi * pi / (LX * LY) * np.cos(pi * x / LX) * np.cos(pi * y / LY)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    m["mu"] = 1e10
    m["eta"] = np.clip(_eta_law(mat, m), opt.etamin, opt.etamax)
    m["exx"] = dvx["x"](X, Y)
    m["eyy"] = dvy["y"](X, Y)
    m["exy"] = 0.5 * (dvx["y"](X, Y) + dvy["x"](X, Y))
    m["sxx"] = 2.0 * m["eta"] * m["exx"]
    m["syy"] = 2.0 * m["eta"] * m["eyy"]
    m["sxy"] = 2.0 * m["eta"] * m["exy"]
    m["p"] = 3300.0 * 9.8 * Y
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    eta_ref = 1e21
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": 3300.0 * 9.8 * YCc,
        "soxx": 2.0 * eta_ref * exx, "soyy": 2.0 * eta_ref * eyy, "soxy": 2.0 * eta_ref * exy,
        "thisT": 273.0 + 1300.0 * np.minimum(1.0, Yb / (0.4 * LY)) + 2.0 * np.sin(pi * Xb / LX) * np.sin(pi * Yb / LY),
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * nodal["soxy"]
    vmax = float(np.max(np.abs(vx))) + float(np.max(np.abs(vy)))
    dmin = min(float(np.min(np.diff(g.x))), float(np.min(np.diff(g.y))))
    dt = 0.5 * dmin / vmax
    return Workload("vep_slab_box", g, m, mat, opt, _free_slip(), nodal, dt, dt, 20)


def periodic_cell_centers(x, LX):
    """getCellCenters then makePeriodic (gridSpacing.c:150-168) for NX lines of a periodic x:
    xc[0..NX+1]."""
    NX = len(x)
    xc = np.empty(NX + 2)
    xc[1:NX] = (x[:-1] + x[1:]) / 2.0
    xc[NX] = (LX + x[NX - 1]) / 2.0
    xc[NX + 1] = xc[1] + LX
    xc[0] = 0.0 - (LX - xc[NX])
    return xc


def periodic_box(nx_cells=16, ny_cells=6, nm=4, seed=9):
    """Visco-elasto-plastic box periodic in x (mechBCLeft/Right type 0 = 2: gridGenerator.c:67-68,
    97-110; nodalFields.c:11-19): nx_cells uniform cells between x = 0 and LX (NX = nx_cells
    lines, line NX = LX is line 0's image), y about 2x finer in the top 20 %, an Arrhenius mantle
    with a Mohr-Coulomb band, and a periodic velocity field with a uniform drift, so markers
    cross x = LX and x = 0 during advection.  Markers on a jittered lattice over [0, LX] x
    [0, LY] plus markers on the periodic seam (X = 0, X = LX, the last cell's halves)."""
    NX, NY = nx_cells, ny_cells + 1
    LX, LY = 4.0e5, 1.0e5
    x = spacing_uniform(0.0, LX, NX + 1)[:NX]
    g = Grid(NX, NY, LX, LY, x, refined_top_y(LY, ny_cells))
    g.xc = periodic_cell_centers(x, LX)[: NX + 1]
    mdx, mdy = LX / (nm * NX), LY / (nm * ny_cells)
    nk, nl = nm * NX, nm * ny_cells
    u = splitmix64_uniform(seed, 2 * nk * nl)
    k = np.repeat(np.arange(nk, dtype=np.float64), nl)
    l = np.tile(np.arange(nl, dtype=np.float64), nk)
    m = np.zeros(nk * nl + 8, dtype=MARKER_DTYPE)
    m["X"][: nk * nl] = mdx * (0.5 + k) + (-mdx / 4.0 + (mdx / 2.0) * u[0::2])
    m["Y"][: nk * nl] = mdy * (0.5 + l) + (-mdy / 4.0 + (mdy / 2.0) * u[1::2])
    xcp = periodic_cell_centers(x, LX)
    seam = [(0.0, 0.3 * LY), (LX, 0.4 * LY), (x[NX - 1], 0.5 * LY), (0.5 * (x[NX - 1] + xcp[NX]), 0.6 * LY),
            (0.5 * (xcp[NX] + LX), 0.7 * LY), (0.5 * xcp[1], 0.2 * LY), (xcp[NX], 0.8 * LY), (LX * (1 - 1e-12), 0.1 * LY)]
    for q, (xx, yy) in enumerate(seam):
        m["X"][nk * nl + q], m["Y"][nk * nl + q] = xx, yy
    m["cellX"] = -1
    m["cellY"] = -1
    X, Y = m["X"], m["Y"]
    ur = splitmix64_uniform(seed + 1000, len(m))
    band = (Y > 0.15 * LY) & (Y < 0.3 * LY)
    m["Mat"] = np.where(band, 1, 0)
    m["T"] = 273.0 + 1300.0 * np.minimum(1.0, Y / (0.4 * LY)) + 5.0 * (ur - 0.5)
    mat = _materials(2)
    for q, (eta, rho) in enumerate([(1e21, 3300.0), (1e23, 3400.0)]):
        mat.materialEta[q] = eta
        mat.materialRho[q] = rho
        mat.materialkThermal[q] = 3.0
        mat.materialCp[q] = 1250.0
        mat.materialAlpha[q] = 3e-5
        mat.materialMu[q] = 1e10
        mat.Tref[q] = 1573.0
    mat.hasEtaT[0] = 1
    mat.QonR[0] = 2.0e4
    mat.hasEtaT[1] = 0
    mat.hasPlasticity[1] = 1
    mat.materialCohesion[1] = 2e7
    mat.materialFriction[1] = 0.6
    opt = Options(etamin=1e19, etamax=1e23, fractionalEtamin=0.1, subgridStressDiffusivity=1.0,
                  subgridTemperatureDiffusivity=1.0)
    pi = np.pi
    kx = 2.0 * pi / LX
    u0, a = 3e-10, 2e-10
    vx_fn = lambda x_, y_: u0 + a * np.sin(kx * x_) * np.cos(pi * y_ / LY)
    vy_fn = lambda x_, y_: -a * (kx * LY / pi) * np.cos(kx * x_) * np.sin(pi * y_ / LY)
    dvx = {"x": lambda x_, y_: a * kx * np.cos(kx * x_) * np.cos(pi * y_ / LY),
           "y": lambda x_, y_: -a * (pi / LY) * np.sin(kx * x_) * np.sin(pi * y_ / LY)}
    dvy = {"x": lambda x_, y_: a * (kx * kx * LY / pi) * np.sin(kx * x_) * np.sin(pi * y_ / LY),
           "y": lambda x_, y_: -a * kx * np.cos(kx * x_) * np.cos(pi * y_ / LY)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    m["mu"] = 1e10
    m["eta"] = np.clip(_eta_law(mat, m), opt.etamin, opt.etamax)
    m["exx"] = dvx["x"](X, Y)
    m["eyy"] = dvy["y"](X, Y)
    m["exy"] = 0.5 * (dvx["y"](X, Y) + dvy["x"](X, Y))
    m["sxx"] = 2.0 * m["eta"] * m["exx"]
    m["syy"] = 2.0 * m["eta"] * m["eyy"]
    m["sxy"] = 2.0 * m["eta"] * m["exy"]
    m["p"] = 3300.0 * 9.8 * Y
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    eta_ref = 1e21
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": 3300.0 * 9.8 * YCc,
        "soxx": 2.0 * eta_ref * exx, "soyy": 2.0 * eta_ref * eyy, "soxy": 2.0 * eta_ref * exy,
        "thisT": 273.0 + 1300.0 * np.minimum(1.0, Yb / (0.4 * LY)) + 2.0 * np.sin(kx * Xb) * np.sin(pi * Yb / LY),
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * nodal["soxy"]
    bcs = _free_slip()
    bcs.mechBCLeft.type[0] = 2
    bcs.mechBCRight.type[0] = 2
    vmax = float(np.max(np.abs(vx))) + float(np.max(np.abs(vy)))
    dmin = min(LX / NX, float(np.min(np.diff(g.y))))
    dt = 0.6 * dmin / vmax
    return Workload("periodic_box", g, m, mat, opt, bcs, nodal, dt, dt, 4)


def ice_creep_box(nx_cells=1024, ny_cells=1024, nm=4, seed=3):
    """Composite ice creep (material law 7): per-marker strain-rate invariant
    10^U[-18,-10] 1/s, T ~ U[100, 273] K, grain size 10^U[-4,-1] m, pressure U[0, 1e8] Pa;
    1025 x 1025 nodes and 16,777,216 markers at full size."""
    NX, NY = nx_cells + 1, ny_cells + 1
    L = 1.0e5
    g = Grid(NX, NY, L, L, spacing_uniform(0.0, L, NX), spacing_uniform(0.0, L, NY))
    m = lattice_markers(g, nm, nm, seed)
    n = len(m)
    u = splitmix64_uniform(seed + 7, 5 * n)
    edot = 10.0 ** (-18.0 + 8.0 * u[0::5])
    phi = 2.0 * np.pi * u[4::5]
    m["exx"] = edot * np.cos(phi)
    m["eyy"] = -m["exx"]
    m["exy"] = edot * np.sin(phi)
    m["T"] = 100.0 + 173.0 * u[1::5]
    grain = 10.0 ** (-4.0 + 3.0 * u[2::5])
    m["p"] = 1e8 * u[3::5]
    mat = _materials(1)
    mat.materialEta[0] = 1e14
    mat.materialRho[0] = 917.0
    mat.materialkThermal[0] = 2.1
    mat.materialCp[0] = 2000.0
    mat.materialAlpha[0] = 1.6e-4
    mat.materialMu[0] = 3.5e9
    mat.hasEtaT[0] = 7
    opt = Options(etamin=1e8, etamax=1e22, fractionalEtamin=0.01, subgridStressDiffusivity=1.0,
                  subgridTemperatureDiffusivity=1.0)
    m["mu"] = 3.5e9
    m["eta"] = 1e14
    m["sxx"] = 2.0 * m["eta"] * m["exx"]
    m["syy"] = 2.0 * m["eta"] * m["eyy"]
    m["sxy"] = 2.0 * m["eta"] * m["exy"]
    U = 1e-9
    pi = np.pi
    vx_fn = lambda x, y: U * np.sin(pi * x / L) * np.cos(pi * y / L)
    vy_fn = lambda x, y: -U * np.cos(pi * x / L) * np.sin(pi * y / L)
    dvx = {"x": lambda x, y: U * pi / L * np.cos(pi * x / L) * np.cos(pi * y / L),
           "y": lambda x, y: -U * pi / L * np.sin(pi * x / L) * np.sin(pi * y / L)}
    dvy = {"x": lambda x, y: U * pi / L * np.sin(pi * x / L) * np.sin(pi * y / L),
           "y": lambda x, y: -U * pi / L * np.cos(pi * x / L) * np.cos(pi * y / L)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    eta_ref = 1e14
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": 1e8 * YCc / L,
        "soxx": 2.0 * eta_ref * exx, "soyy": 2.0 * eta_ref * eyy, "soxy": 2.0 * eta_ref * exy,
        "thisT": 100.0 + 173.0 * Yb / L,
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * nodal["soxy"]
    dt = 0.5 * (L / nx_cells) / (2 * U)
    wl = Workload("ice_creep_box", g, m, mat, opt, _free_slip(), nodal, dt, dt, 10)
    wl.grain_size = grain
    return wl


def convection_member(nx_cells, ny_cells, nmx, nmy, Ra, contrast, seed):
    """One ensemble member: thermal convection in a box of aspect nx_cells:ny_cells (height 1),
    viscosity exp(-ln(contrast) T) (hasEtaT 5), free slip, T0 = 1 - y + 0.01 cos(pi x) sin(pi y);
    prescribed cellular flow with speed 100 (Ra / 1e4)^(2/3).  No host markers: the member's
    markers are laid out on the device (resetMarkers, distributeMarkersUniformInDomain with
    nmx x nmy per cell and this seed, Mat 0, T from the nodal field, viscosity from T)."""
    NX, NY = nx_cells + 1, ny_cells + 1
    LX = float(nx_cells) / float(ny_cells)
    g = Grid(NX, NY, LX, 1.0, spacing_uniform(0.0, LX, NX), spacing_uniform(0.0, 1.0, NY))
    mat = _materials(1)
    mat.materialEta[0] = 1.0
    mat.materialRho[0] = 1.0
    mat.materialkThermal[0] = 1.0
    mat.materialCp[0] = 1.0
    mat.materialAlpha[0] = 1.0
    mat.materialMu[0] = 1e20
    mat.hasEtaT[0] = 5
    mat.QonR[0] = math.log(contrast)
    mat.Tref[0] = 1.0
    opt = Options(etamin=1.0 / contrast, etamax=contrast, fractionalEtamin=0.01, subgridStressDiffusivity=0.0,
                  subgridTemperatureDiffusivity=1.0)
    U = 100.0 * (Ra / 1e4) ** (2.0 / 3.0)
    pi = np.pi
    vx_fn = lambda x, y: U * pi * np.sin(pi * x / LX) * np.cos(pi * y)
    vy_fn = lambda x, y: -U * pi / LX * np.cos(pi * x / LX) * np.sin(pi * y)
    dvx = {"x": lambda x, y: U * pi * pi / LX * np.cos(pi * x / LX) * np.cos(pi * y),
           "y": lambda x, y: -U * pi * pi * np.sin(pi * x / LX) * np.sin(pi * y)}
    dvy = {"x": lambda x, y: U * pi * pi / LX ** 2 * np.sin(pi * x / LX) * np.sin(pi * y),
           "y": lambda x, y: -U * pi * pi / LX * np.cos(pi * x / LX) * np.cos(pi * y)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    Tn = 1.0 - Yb + 0.01 * np.cos(pi * Xb / LX) * np.sin(pi * Yb)
    eta_c = np.exp(-math.log(contrast) * np.clip(1.0 - YCc, 0.0, 1.0))
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": np.zeros((NY, NX)),
        "soxx": 2.0 * eta_c * exx, "soyy": 2.0 * eta_c * eyy, "soxy": np.zeros((NY, NX)),
        "thisT": Tn + 1e-3 * np.sin(pi * Xb / LX) * np.sin(pi * Yb), "lastT": Tn,
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * exy
    dt = 0.5 * (1.0 / ny_cells) / (U * pi)
    wl = Workload("convection_member", g, np.zeros(0, dtype=MARKER_DTYPE), mat, opt, _free_slip(), nodal, dt, dt,
                  10)
    wl.nm = (nmx, nmy)
    wl.seed = seed
    wl.capacity = nmx * nmy * nx_cells * ny_cells
    return wl


def convection_ensemble(n_members=64, seed=4):
    """Ensemble of independent convection runs: square grids drawn from {64^2, 128^2, 256^2,
    512^2} cells, 9, 16 or 25 markers per cell (3x3, 4x4, 5x5), Ra log-uniform in [1e4, 1e7],
    viscosity contrast log-uniform in [1e1, 1e5]; all draws from SplitMix64(seed)."""
    u = splitmix64_uniform(seed, 4 * n_members)
    members = []
    for i in range(n_members):
        ncell = (64, 128, 256, 512)[min(3, int(u[4 * i] * 4))]
        nm = (3, 4, 5)[min(2, int(u[4 * i + 1] * 3))]
        Ra = 10 ** (4 + 3 * u[4 * i + 2])
        contrast = 10 ** (1 + 4 * u[4 * i + 3])
        members.append(convection_member(ncell, ncell, nm, nm, Ra, contrast, seed * 1000 + i))
    return members


def ice_member(nx_cells, ny_cells, seed, nm=4):
    """One member of the mixed ice ensemble: the composite-creep (law 7) visco-elasto-plastic
    box of ice_creep_box on an nx_cells x ny_cells grid (100 km wide, aspect as given), with
    Drucker-Prager yield (cohesion 1 MPa, friction 0.6) and shear modulus 3.5 GPa.  No host
    markers: nm x nm markers per cell are laid out on the device; grain sizes (log10 d ~
    U[-4,-1] m, SplitMix64) follow in distribution order."""
    NX, NY = nx_cells + 1, ny_cells + 1
    LX = 1.0e5
    LY = LX * ny_cells / nx_cells
    g = Grid(NX, NY, LX, LY, spacing_uniform(0.0, LX, NX), spacing_uniform(0.0, LY, NY))
    mat = _materials(1)
    mat.materialEta[0] = 1e14
    mat.materialRho[0] = 917.0
    mat.materialkThermal[0] = 2.1
    mat.materialCp[0] = 2000.0
    mat.materialAlpha[0] = 1.6e-4
    mat.materialMu[0] = 3.5e9
    mat.hasEtaT[0] = 7
    mat.hasPlasticity[0] = 1
    mat.materialCohesion[0] = 1e6
    mat.materialFriction[0] = 0.6
    opt = Options(etamin=1e8, etamax=1e22, fractionalEtamin=0.01, subgridStressDiffusivity=1.0,
                  subgridTemperatureDiffusivity=1.0)
    U = 1e-9
    pi = np.pi
    vx_fn = lambda x, y: U * np.sin(pi * x / LX) * np.cos(pi * y / LY)
    vy_fn = lambda x, y: -U * LY / LX * np.cos(pi * x / LX) * np.sin(pi * y / LY)
    dvx = {"x": lambda x, y: U * pi / LX * np.cos(pi * x / LX) * np.cos(pi * y / LY),
           "y": lambda x, y: -U * pi / LY * np.sin(pi * x / LX) * np.sin(pi * y / LY)}
    dvy = {"x": lambda x, y: U * pi * LY / LX ** 2 * np.sin(pi * x / LX) * np.sin(pi * y / LY),
           "y": lambda x, y: -U * pi / LX * np.cos(pi * x / LX) * np.cos(pi * y / LY)}
    vx, vy, exx, eyy, exy, wxy = _velocity_fields(g, vx_fn, vy_fn, dvx, dvy)
    XCc, YCc = np.meshgrid(g.xc[:NX], g.yc[:NY], indexing="xy")
    Xb, Yb = np.meshgrid(g.x, g.y, indexing="xy")
    eta_ref = 1e14
    nodal = {
        "vx": vx, "vy": vy, "edotxx": exx, "edotyy": eyy, "edotxy": exy, "wxy": wxy,
        "p": 1e8 * YCc / LY,
        "soxx": 2.0 * eta_ref * exx, "soyy": 2.0 * eta_ref * eyy, "soxy": 2.0 * eta_ref * exy,
        "thisT": 100.0 + 173.0 * Yb / LY, "lastT": 100.0 + 173.0 * Yb / LY,
    }
    nodal["dsxx"] = 0.05 * nodal["soxx"]
    nodal["dsyy"] = 0.05 * nodal["soyy"]
    nodal["dsxy"] = 0.05 * nodal["soxy"]
    dt = 0.5 * (LX / nx_cells) / (2 * U)
    wl = Workload("ice_member", g, np.zeros(0, dtype=MARKER_DTYPE), mat, opt, _free_slip(), nodal, dt, dt, 10)
    wl.nm = (nm, nm)
    wl.seed = seed
    wl.capacity = nm * nm * nx_cells * ny_cells
    return wl


def ice_grain_sizes(n, seed):
    return 10.0 ** (-4.0 + 3.0 * splitmix64_uniform(seed + 17, n))


# mixed member grids (cells) and their draw probabilities: most members small, a few at the
# 1024 x 256 size of the VEP box
ICE_GRIDS = [(128, 128), (256, 64), (128, 256), (192, 192), (1024, 256)]
ICE_GRID_P = [0.55, 0.25, 0.12, 0.075, 0.005]


def ice_ensemble(n_members=256, seed=5):
    """Ensemble of independent ice-creep VEP boxes on mixed grids from 128^2 to 1024 x 256 cells,
    16 markers per cell (SplitMix64 seed 5): about 80-90 million markers."""
    u = splitmix64_uniform(seed, n_members)
    cum = np.cumsum(ICE_GRID_P)
    out = []
    for i in range(n_members):
        nx, ny = ICE_GRIDS[min(len(ICE_GRIDS) - 1, int(np.searchsorted(cum, u[i], side="right")))]
        out.append(ice_member(nx, ny, seed * 1000 + i))
    return out


def density_case(nx_cells=32, ny_cells=8, seed=6):
    """A marker set for checkMarkerDensity (markers.c:455-781): the refined VEP box at 4x4
    markers per cell (4 per quarter cell) with quarter cells emptied (including some in the first
    cell column, where the reference creates slab-inflow markers, and in the last column below
    the overriding plate, where it creates mantle-inflow markers) and quarter cells overfilled
    with markers moved in from elsewhere.  Returns (workload, density options) for
    minMarkers = 1 (the reference default), maxMarkers = 6 and NMX = NMY = 8 (its quarter-cell
    target ceil(NMX (NX-1)/2 dx/LX) with dx half a cell width is NMX/4 per axis)."""
    from .mic_types import DensityOptions

    wl = vep_slab_box(nx_cells=nx_cells, ny_cells=ny_cells, nm=4, seed=seed)
    g, m = wl.grid, wl.markers
    u = splitmix64_uniform(seed + 100, 4096)
    xc = cell_centers(g.x, g.LX)
    yc = cell_centers(g.y, g.LY)

    def quarter(i, j):  # bounds of basic quarter cell (i, j) as the reference computes them
        xmin = g.x[i // 2] if i % 2 == 0 else xc[(i + 1) // 2]
        xmax = xc[i // 2 + 1] if i % 2 == 0 else g.x[(i + 1) // 2]
        ymin = g.y[j // 2] if j % 2 == 0 else yc[(j + 1) // 2]
        ymax = yc[j // 2 + 1] if j % 2 == 0 else g.y[(j + 1) // 2]
        return xmin, xmax, ymin, ymax

    def inside(b):
        return (m["X"] >= b[0]) & (m["X"] < b[1]) & (m["Y"] >= b[2]) & (m["Y"] < b[3])

    nqx, nqy = 2 * nx_cells, 2 * ny_cells
    empty = [(0, 1), (1, nqy - 2), (5, 3), (nqx - 1, nqy - 1), (nqx - 2, nqy - 3), (nqx // 2, nqy // 2),
             (nqx // 2 + 1, nqy // 2)]
    for (i, j) in empty:
        m["X"][inside(quarter(i, j))] = -1.0  # leave the domain: out-of-domain markers
    full = [(3, 4), (nqx // 3, 2), (nqx - 5, nqy // 2 + 1)]
    donors = np.flatnonzero(m["X"] > 0)[::7]
    k = 0
    for n_extra, (i, j) in zip((5, 9, 3), full):
        b = quarter(i, j)
        for e in range(n_extra):
            d = donors[k]
            m["X"][d] = b[0] + (b[1] - b[0]) * (0.05 + 0.9 * u[2 * k])
            m["Y"][d] = b[2] + (b[3] - b[2]) * (0.05 + 0.9 * u[2 * k + 1])
            k += 1
    dopt = DensityOptions(NMX=8, NMY=8, minMarkers=1, maxMarkers=6, slabAngle=0.5, slabAge=50.0,
                          overridingPlateThickness=0.3 * g.LY, rootThickness=0.05 * g.LY, rootCenter=0.9 * g.LX,
                          rootWidth=0.2 * g.LX)
    return wl, dopt


def subduction_box(nx_cells=128, ny_cells=32, nm=4, seed=4):
    """The refined VEP box as a self-consistent subduction model: markers nm x nm per cell, a slab
    dipping at 0.8 rad entering from the left at 5 cm/yr below an overriding plate 0.3 LY thick
    (with a root 0.05 LY deep centred at LX/2), gravity 10 m/s^2, top at 273 K.  Returns
    (workload, mic_timestep_options) for mic_subduction_timestep: first step, at most 4
    plasticity iterations, displacement limit half a cell, temperature change limit 50 K."""
    from .mic_types import DensityOptions, SubductionOptions, TimestepOptions

    wl = vep_slab_box(nx_cells=nx_cells, ny_cells=ny_cells, nm=nm, seed=seed)
    g = wl.grid
    so = SubductionOptions(gx=0.0, gy=10.0, slabVelocity=0.05 / 3.15576e7, slabAngle=0.8, slabAge=50.0,
                           overridingPlateThickness=0.3 * g.LY, rootThickness=0.05 * g.LY, rootCenter=0.5 * g.LX,
                           rootWidth=0.2 * g.LX, thermalBCTopType=0, thermalBCTopValue=273.0)
    topt = TimestepOptions(dtMax=3.0e11, displacementStepLimit=0.5, maxTempChange=50.0, maxNumPlasticity=4,
                           shearHeating=1, firstStep=1, densityControl=0,
                           density=DensityOptions(NMX=nm, NMY=nm, minMarkers=1, maxMarkers=100), sub=so,
                           thermalBCBottomValue=1573.0)
    return wl, topt


WORKLOADS = {
    "convection_box": convection_box,
    "vep_slab_box": vep_slab_box,
    # 513 x 129 nodes, 1,048,576 markers (about 220 MB of marker state, larger than L2):
    # the small case used for detailed profiles
    "vep_slab_box_1m": lambda: vep_slab_box(nx_cells=512, ny_cells=128),
    "ice_creep_box": ice_creep_box,
    # 513 x 513 nodes, 4,194,304 markers
    "ice_creep_box_4m": lambda: ice_creep_box(nx_cells=512, ny_cells=512),
    # 129 x 129 nodes, 262,144 markers with the ice box's per-marker distributions: the bounded
    # sample the host-core baseline steps
    "ice_creep_box_sample": lambda: ice_creep_box(nx_cells=128, ny_cells=128),
    "vep_slab_box_sample": lambda: vep_slab_box(nx_cells=256, ny_cells=64),
}
