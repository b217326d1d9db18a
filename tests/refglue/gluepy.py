"""ctypes driver for the reference-side binding (tests/refglue/glue_driver.c over
fvmic2d_gb300/refglue/fvmic2d_glue.c).  TEST INFRASTRUCTURE ONLY.  GlueProblem has the surface
of oracle.oraclepy.OracleProblem, so the same entry-point sequences run through fvmic2d's own
routine names (the binding) and through the oracle."""
import ctypes

import numpy as np

from fvmic2d_gb300.mic_types import MARKER_DTYPE, MARKER_F64_OFFSETS, NF

from . import build

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)

_libs = {}

SIGS = {
    "gd_create": (_P, [_I, _I, _D, _D, _DP, _DP, _I]),
    "gd_destroy": (None, [_P]),
    "gd_set_materials": (None, [_P, _P]),
    "gd_set_bcs": (None, [_P, _P]),
    "gd_set_options": (None, [_P, _P]),
    "gd_set_markers": (_I, [_P, _P, _I]),
    "gd_get_markers": (_I, [_P, _P, _I]),
    "gd_marker_count": (_I, [_P]),
    "gd_set_nodal": (_I, [_P, _I, _DP]),
    "gd_get_nodal": (_I, [_P, _I, _DP]),
    "gd_last_error": (_I, []),
    "gd_resetMarkers": (None, [_P]),
    "gd_distributeMarkersUniformInDomain": (_I, [_P, _I, _I]),
    "gd_findMarkerCells": (_I, [_P]),
    "gd_updateMarkerRho": (_I, [_P]),
    "gd_maxMarkerT": (_D, [_P]),
    "gd_maxAbsSxx": (_D, [_P]),
    "gd_projectMarkersNodesAll2": (_I, [_P]),
    "gd_projectMarkerFieldToNodes": (_I, [_P, _I, _DP, _I, _I, _I, _I]),
    "gd_projectNodalFieldToMarkersS": (_I, [_P, _I, _I]),
    "gd_projectMarkersNodesFromScalar": (_I, [_P, _DP, _I]),
    "gd_checkPlasticYielding": (_I, [_P, _D, _D]),
    "gd_limitViscosity": (None, [_P]),
    "gd_updateViscosity": (None, [_P]),
    "gd_updateMarkerStrainPressure": (_I, [_P, _D]),
    "gd_updateGlobalStrainRateResidual": (_D, [_P, _I]),
    "gd_setGlobalStrainRateResidual": (None, [_I, _D]),
    "gd_checkConvergence": (_I, [_D, _D, _I]),
    "gd_subgridStressChanges": (_I, [_P, _D, _D]),
    "gd_updateMarkerStress": (_I, [_P]),
    "gd_subgridTemperatureChanges": (_I, [_P, _D]),
    "gd_advectMarkersRK": (_I, [_P, _D]),
    "gd_checkMarkerDensity": (_I, [_P, _P]),
}


def lib(exact=False):
    if exact not in _libs:
        L = ctypes.CDLL(build.build_driver(exact))
        for name, (res, args) in SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[exact] = L
    return _libs[exact]


def _dp(a):
    return a.ctypes.data_as(_DP)


class GlueError(RuntimeError):
    pass


class GlueProblem:
    """One grid and one MarkerSet driven through the binding.  The binding keeps one marker set
    per process (its device context), so only one GlueProblem may be alive at a time."""

    def __init__(self, wl, markers=None, capacity=None, exact=False):
        L = self.L = lib(exact)
        g = wl.grid
        self.wl = wl
        self.NX, self.NY = g.NX, g.NY
        mk = np.ascontiguousarray(wl.markers if markers is None else markers, dtype=MARKER_DTYPE)
        cap = capacity or max(len(mk), 1)
        self.h = L.gd_create(g.NX, g.NY, g.LX, g.LY, _dp(np.ascontiguousarray(g.x, dtype=np.float64)),
                             _dp(np.ascontiguousarray(g.y, dtype=np.float64)), cap)
        if not self.h:
            raise GlueError("gd_create failed")
        self.cap = cap
        self.materials, self.options, self.bcs = wl.materials, wl.options, wl.bcs
        L.gd_set_materials(self.h, ctypes.byref(self.materials))
        L.gd_set_options(self.h, ctypes.byref(self.options))
        L.gd_set_bcs(self.h, ctypes.byref(self.bcs))
        if len(mk):
            self._check(L.gd_set_markers(self.h, mk.ctypes.data, len(mk)), "set markers")
        for name, arr in wl.nodal.items():
            self.set_nodal(name, arr)

    def _check(self, code, what):
        if code:
            raise GlueError("%s failed: %d (last library error %d)" % (what, code, self.L.gd_last_error()))

    def close(self):
        if getattr(self, "h", None):
            self.L.gd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        return self.L.gd_marker_count(self.h)

    @property
    def markers(self):
        out = np.zeros(max(self.n, 0), dtype=MARKER_DTYPE)
        n = self.L.gd_get_markers(self.h, out.ctypes.data, len(out))
        if n < 0:
            raise GlueError("markers to host failed")
        return out

    def set_nodal(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.NY, self.NX)
        self._check(self.L.gd_set_nodal(self.h, NF[name], _dp(a)), "set nodal " + name)

    def get_nodal(self, name):
        a = np.empty((self.NY, self.NX))
        self._check(self.L.gd_get_nodal(self.h, NF[name], _dp(a)), "get nodal " + name)
        return a

    # ---- fvmic2d's routines, by their own names --------------------------------------
    def resetMarkers(self):
        self.L.gd_resetMarkers(self.h)

    def distributeMarkersUniformInDomain(self, NMX, NMY):
        n = self.L.gd_distributeMarkersUniformInDomain(self.h, NMX, NMY)
        if n < 0:
            raise GlueError("distributeMarkersUniformInDomain failed")
        return n

    def findMarkerCells(self):
        nout = self.L.gd_findMarkerCells(self.h)
        self._check(self.L.gd_last_error(), "findMarkerCells")
        return nout

    def updateMarkerRho(self):
        self._check(self.L.gd_updateMarkerRho(self.h), "density update")

    def maxMarkerT(self):
        return self.L.gd_maxMarkerT(self.h)

    def maxAbsSxx(self):
        return self.L.gd_maxAbsSxx(self.h)

    def projectMarkersNodesAll2(self):
        self._check(self.L.gd_projectMarkersNodesAll2(self.h), "projectMarkersNodesAll2")

    def projectMarkerFieldToNodes(self, field, out, stagx, stagy, method, matprop=None):
        off = -1 if field is None else MARKER_F64_OFFSETS[field]
        mp = None if matprop is None else _dp(np.ascontiguousarray(matprop, dtype=np.float64))
        self._check(self.L.gd_projectMarkerFieldToNodes(self.h, off, mp, NF[out], stagx, stagy, method),
                    "projectMarkerFieldToNodes")

    def projectNodalFieldToMarkersS(self, nodal, field):
        self._check(self.L.gd_projectNodalFieldToMarkersS(self.h, NF[nodal], MARKER_F64_OFFSETS[field]),
                    "projectNodalFieldToMarkersS")

    def projectMarkersNodesFromScalar(self, values, nodal):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.L.gd_projectMarkersNodesFromScalar(self.h, _dp(v), NF[nodal]), "projectMarkersNodesFromScalar")

    def checkPlasticYielding(self, dt, t=0.0):
        y = self.L.gd_checkPlasticYielding(self.h, dt, t)
        if y < 0:
            raise GlueError("checkPlasticYielding failed (%d)" % self.L.gd_last_error())
        return y

    def limitViscosity(self):
        self.L.gd_limitViscosity(self.h)

    def updateViscosity(self):
        self.L.gd_updateViscosity(self.h)

    def updateMarkerStrainPressure(self, dt):
        self._check(self.L.gd_updateMarkerStrainPressure(self.h, dt), "updateMarkerStrainPressure")

    def updateGlobalStrainRateResidual(self, it):
        return self.L.gd_updateGlobalStrainRateResidual(self.h, it)

    def setGlobalStrainRateResidual(self, it, v):
        self.L.gd_setGlobalStrainRateResidual(it, v)

    def checkConvergence(self, atol, rtol, it):
        return self.L.gd_checkConvergence(atol, rtol, it)

    def subgridStressChanges(self, dt, D):
        self._check(self.L.gd_subgridStressChanges(self.h, dt, D), "subgridStressChanges")

    def updateMarkerStress(self):
        self._check(self.L.gd_updateMarkerStress(self.h), "updateMarkerStress")

    def subgridTemperatureChanges(self, dt):
        self._check(self.L.gd_subgridTemperatureChanges(self.h, dt), "subgridTemperatureChanges")

    def advectMarkersRK(self, dt):
        self._check(self.L.gd_advectMarkersRK(self.h, dt), "advectMarkersRK")

    def checkMarkerDensity(self, dopt):
        """dopt: fvmic2d_gb300.mic_types.DensityOptions"""
        n = self.L.gd_checkMarkerDensity(self.h, ctypes.byref(dopt))
        if n < 0:
            raise GlueError("checkMarkerDensity failed (%d)" % self.L.gd_last_error())
        return n
