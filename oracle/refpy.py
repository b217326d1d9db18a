"""ctypes driver for oracle/_ref/libfvmic2d_ref.so: fvmic2d's own hot-path C compiled
against petsc_lite (oracle/build_ref.sh).  TEST INFRASTRUCTURE ONLY: pins the C
restatement (oracle/mic_oracle.c) and generates tests/golden/ fixtures.  The
library only exists where the reference tree is present (never on the GPU machine)."""
import ctypes
import os

import numpy as np

from fvmic2d_gb300.mic_types import NF, MARKER_DTYPE, MARKER_F64_OFFSETS

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libfvmic2d_ref.so")
# the same sources with markers.c compiled under -DJAUMANN (the Jaumann stress rotation of
# advectMarkersRK, markers.c:2147-2156)
LIB_PATH_JAUMANN = os.path.join(HERE, "_ref", "libfvmic2d_ref_jaumann.so")

_libs = {}
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)


def available(jaumann=False):
    return os.path.exists(LIB_PATH_JAUMANN if jaumann else LIB_PATH)


def lib(jaumann=False):
    if jaumann not in _libs:
        path = LIB_PATH_JAUMANN if jaumann else LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError("%s missing: run oracle/build_ref.sh where the reference tree exists" % path)
        L = ctypes.CDLL(path)
        sig = {
            "ref_create": (_P, [_I, _I, _D, _D, _DP, _DP]),
            "ref_destroy": (None, [_P]),
            "ref_get_grid": (None, [_P, _DP, _DP]),
            "ref_set_materials": (None, [_P, _P]),
            "ref_set_bcs": (None, [_P, _P]),
            "ref_set_periodic_x": (None, [_P]),
            "ref_set_options": (None, [_P, _P]),
            "ref_set_markers": (None, [_P, _P, _I]),
            "ref_set_nodal": (_I, [_P, _I, _DP]),
            "ref_get_nodal": (_I, [_P, _I, _DP]),
            "ref_findMarkerCells": (_I, [_P]),
            "ref_updateMarkerRho": (None, [_P]),
            "ref_maxMarkerT": (_D, [_P]),
            "ref_maxAbsSxx": (_D, [_P]),
            "ref_projectMarkersNodesAll2": (_I, [_P]),
            "ref_projectMarkerFieldToNodes": (_I, [_P, _I, _DP, _I, _I, _I, _I]),
            "ref_projectNodalFieldToMarkersS": (_I, [_P, _I, _I]),
            "ref_checkPlasticYielding": (_I, [_P, _D, _D]),
            "ref_limitViscosity": (None, [_P]),
            "ref_updateViscosity": (None, [_P]),
            "ref_updateMarkerStrainPressure": (_I, [_P, _D]),
            "ref_updateGlobalStrainRateResidual": (_D, [_P, _I]),
            "ref_checkConvergence": (_I, [_D, _D, _I]),
            "ref_subgridStressChanges": (_I, [_P, _D, _D]),
            "ref_updateMarkerStress": (_I, [_P]),
            "ref_subgridTemperatureChanges": (_I, [_P, _D]),
            "ref_advectMarkersRK": (_I, [_P, _D]),
            "ref_goldsbyKohlstedt": (_D, [_D, _D, _D, _D]),
            "ref_goldsbyKohlstedt_many": (None, [_DP, _DP, _DP, _DP, _DP, _I]),
            "ref_resetMarkers": (_I, [_P, _P, _I]),
            "ref_checkMarkerDensity": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _DP, ctypes.c_long,
                                            ctypes.POINTER(ctypes.c_ushort)]),
            "ref_distributeMarkersUniformInDomain": (_I, [_P, _P, _I, _I, _I]),
            "ref_nodalStressStrain": (_I, [_P, _D, _D]),
            "ref_projectMarkersNodesFromScalar": (_I, [_P, _DP, _I]),
            "ref_saveMarkersBinary": (_I, [_P, _P, _I, _I, _I, _D]),
            "ref_restartFromMarkers": (_I, [_P, _I, _I, _D, _P, _I, _DP]),
            "ref_limitDisplacementTimestep": (_D, [_P, _D, _D]),
            "ref_retrieveSolutions": (_I, [_P, _DP, _D]),
            "ref_formVEPSystem": (_I, [_P, _P, _D, _DP, _DP]),
            "ref_adiabaticHeating": (_I, [_P, _D]),
            "ref_initialConditionsVanKeken": (_I, [_P, _P, _I, _P, _P]),
            "ref_nusseltNumber": (_D, [_P, _D, _D]),
            "ref_rmsVelocity": (_D, [_P]),
            "ref_enforceThermalBCs1": (_I, [_P, _P]),
            "ref_formThermalSystem": (_I, [_P, _P, _D, _I]),
            "ref_system_nnz": (ctypes.c_long, [_I, ctypes.POINTER(ctypes.c_long)]),
            "ref_system_get": (None, [_I, _P, _P, _DP, _DP]),
            "ref_stage_seconds": (_D, [_I]),
            "ref_stage_reset": (None, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[jaumann] = L
    return _libs[jaumann]


def _dp(a):
    return a.ctypes.data_as(_DP)


class RefProblem:
    """One reference problem: grid + nodal Vecs + material/option tables + a marker array
    that stays owned by this object (the reference functions mutate it in place)."""

    def __init__(self, wl, markers=None, jaumann=False):
        """jaumann: step with the reference built under -DJAUMANN"""
        self.L = L = lib(jaumann)
        g = wl.grid
        self.wl = wl
        self.NX, self.NY = g.NX, g.NY
        self.h = L.ref_create(g.NX, g.NY, g.LX, g.LY, _dp(g.x), _dp(g.y))
        self.materials = wl.materials
        self.options = wl.options
        self.bcs = wl.bcs
        L.ref_set_materials(self.h, ctypes.byref(self.materials))
        L.ref_set_options(self.h, ctypes.byref(self.options))
        L.ref_set_bcs(self.h, ctypes.byref(self.bcs))
        if self.bcs.mechBCLeft.type[0] == 2 or self.bcs.mechBCRight.type[0] == 2:
            L.ref_set_periodic_x(self.h)  # nodalFields.c:11-19, gridGenerator.c:67-68
        self.markers = np.array(wl.markers if markers is None else markers, dtype=MARKER_DTYPE, copy=True)
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        for name, arr in wl.nodal.items():
            self.set_nodal(name, arr)

    def saveMarkersBinary(self, iMonte, iTime, elapsed_time):
        """writes output/Markers.<iMonte>.<iTime> under the current directory"""
        L = self.L
        e = L.ref_saveMarkersBinary(self.h, self.markers.ctypes.data, len(self.markers), iMonte, iTime, elapsed_time)
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        return e

    def restartFromMarkers(self, iMonte, iTime, cap, maxMarkFactor=1.0):
        L = self.L
        mk = np.zeros(cap, dtype=self.markers.dtype)
        t = ctypes.c_double(0.0)
        n = L.ref_restartFromMarkers(self.h, iMonte, iTime, maxMarkFactor, mk.ctypes.data, cap, ctypes.byref(t))
        if n < 0:
            raise IOError("restartFromMarkers failed")
        self.markers = mk[:n].copy()
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        return t.value

    def projectMarkersNodesFromScalar(self, values, nodal):
        v = np.ascontiguousarray(values, dtype=np.float64)
        return self.L.ref_projectMarkersNodesFromScalar(self.h, _dp(v), NF[nodal])

    def nodalStressStrain(self, dt, gy=0.0):
        return self.L.ref_nodalStressStrain(self.h, dt, gy)

    def limitDisplacementTimestep(self, dt, factor):
        return self.L.ref_limitDisplacementTimestep(self.h, dt, factor)

    def retrieveSolutions(self, S, Kcont):
        S = np.ascontiguousarray(S, dtype=np.float64)
        return self.L.ref_retrieveSolutions(self.h, _dp(S), Kcont)

    def _system(self, which):
        L = self.L
        nrows = ctypes.c_long(0)
        nnz = L.ref_system_nnz(which, ctypes.byref(nrows))
        rowptr = np.zeros(nrows.value + 1, dtype=np.int32)
        cols = np.zeros(max(nnz, 1), dtype=np.int32)
        vals = np.zeros(max(nnz, 1), dtype=np.float64)
        rhs = np.zeros(nrows.value, dtype=np.float64)
        L.ref_system_get(which, rowptr.ctypes.data, cols.ctypes.data, _dp(vals), _dp(rhs))
        return rowptr, cols[:nnz], vals[:nnz], rhs

    def formVEPSystem(self, sopt, dt):
        """formVEPSystem (vep_system.c:12) on the nodal fields: (rowptr, cols, vals, rhs, Kbond,
        Kcont), the matrix as CSR with ascending columns, rows in the reference's ordering
        3 (j NX + i) + dof"""
        kb, kc = ctypes.c_double(0.0), ctypes.c_double(0.0)
        e = self.L.ref_formVEPSystem(self.h, ctypes.byref(sopt), dt, ctypes.byref(kb), ctypes.byref(kc))
        if e:
            raise RuntimeError("formVEPSystem failed: %d" % e)
        return self._system(0) + (kb.value, kc.value)

    def adiabaticHeating(self, gy):
        """adiabaticHeating (adiabaticHeating.c:7) added to the heating field as main adds it"""
        e = self.L.ref_adiabaticHeating(self.h, gy)
        if e:
            raise RuntimeError("adiabaticHeating failed: %d" % e)

    def nusseltNumber(self, bottom, top):
        return self.L.ref_nusseltNumber(self.h, bottom, top)

    def rmsVelocity(self):
        return self.L.ref_rmsVelocity(self.h)

    def initialConditionsVanKeken(self, sopt):
        """initialConditionsVanKeken on this problem's markers; returns the BCs it sets"""
        from fvmic2d_gb300.mic_types import BCs

        b = BCs()
        e = self.L.ref_initialConditionsVanKeken(self.h, self.markers.ctypes.data, len(self.markers),
                                                ctypes.byref(sopt), ctypes.byref(b))
        self.L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        if e:
            raise RuntimeError("initialConditionsVanKeken failed: %d" % e)
        return b

    def enforceThermalBCs1(self, sopt):
        e = self.L.ref_enforceThermalBCs1(self.h, ctypes.byref(sopt))
        if e:
            raise RuntimeError("enforceThermalBCs1 failed: %d" % e)

    def formThermalSystem(self, sopt, dt, doSteady=0):
        """formThermalSystem (formThermalSystem.c:6) with the right-hand side starting as the
        heating field: (rowptr, cols, vals, rhs)"""
        e = self.L.ref_formThermalSystem(self.h, ctypes.byref(sopt), dt, doSteady)
        if e:
            raise RuntimeError("formThermalSystem failed: %d" % e)
        return self._system(1)

    def checkMarkerDensity(self, dopt, cap, seed=1):
        """The reference's checkMarkerDensity (PETSCRAND48 object seeded with srand48(seed)) on a
        copy of the markers grown to capacity cap; returns (markers[:n_new], 48-bit state)."""
        L = self.L
        mk = np.zeros(cap, dtype=self.markers.dtype)
        mk[:len(self.markers)] = self.markers
        slab = np.array([dopt.slabAngle, dopt.slabAge, dopt.overridingPlateThickness, dopt.rootThickness,
                         dopt.rootCenter, dopt.rootWidth])
        st = (ctypes.c_ushort * 3)()
        n = L.ref_checkMarkerDensity(self.h, mk.ctypes.data, len(self.markers), cap, dopt.NMX, dopt.NMY,
                                     dopt.minMarkers, dopt.maxMarkers, _dp(slab), seed, st)
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        if n < 0:
            raise RuntimeError("checkMarkerDensity failed")
        self.markers = mk[:n].copy()
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        state = int(st[0]) | (int(st[1]) << 16) | (int(st[2]) << 32)
        return self.markers, state

    def distribute_uniform(self, NMX, NMY, cap=None):
        """The reference's resetMarkers + distributeMarkersUniformInDomain (seed 0)."""
        L = self.L
        cap = cap or NMX * NMY * (self.wl.grid.NX - 1) * (self.wl.grid.NY - 1) + 16
        mk = np.zeros(cap, dtype=self.markers.dtype)
        L.ref_resetMarkers(self.h, mk.ctypes.data, cap)
        n = L.ref_distributeMarkersUniformInDomain(self.h, mk.ctypes.data, cap, NMX, NMY)
        L.ref_set_markers(self.h, self.markers.ctypes.data, len(self.markers))
        return mk, n

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid_centres(self):
        xc = np.empty(self.NX + 1)
        yc = np.empty(self.NY + 1)
        self.L.ref_get_grid(self.h, _dp(xc), _dp(yc))
        return xc, yc

    def set_nodal(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.NY, self.NX)
        assert self.L.ref_set_nodal(self.h, NF[name], _dp(a)) == 0

    def get_nodal(self, name):
        a = np.empty((self.NY, self.NX))
        assert self.L.ref_get_nodal(self.h, NF[name], _dp(a)) == 0
        return a

    # --- reference entry points -------------------------------------------------
    def findMarkerCells(self):
        return self.L.ref_findMarkerCells(self.h)

    def updateMarkerRho(self):
        self.L.ref_updateMarkerRho(self.h)

    def maxMarkerT(self):
        return self.L.ref_maxMarkerT(self.h)

    def maxAbsSxx(self):
        return self.L.ref_maxAbsSxx(self.h)

    def projectMarkersNodesAll2(self):
        return self.L.ref_projectMarkersNodesAll2(self.h)

    def projectMarkerFieldToNodes(self, field, out, stagx, stagy, method, matprop=None):
        off = -1 if field is None else MARKER_F64_OFFSETS[field]
        mp = None
        if matprop is not None:
            self._mp = np.ascontiguousarray(matprop, dtype=np.float64)
            mp = _dp(self._mp)
        return self.L.ref_projectMarkerFieldToNodes(self.h, off, mp, NF[out], stagx, stagy, method)

    def projectNodalFieldToMarkersS(self, nodal, field):
        return self.L.ref_projectNodalFieldToMarkersS(self.h, NF[nodal], MARKER_F64_OFFSETS[field])

    def checkPlasticYielding(self, dt, t=0.0):
        return self.L.ref_checkPlasticYielding(self.h, dt, t)

    def limitViscosity(self):
        self.L.ref_limitViscosity(self.h)

    def updateMarkerStrainPressure(self, dt):
        return self.L.ref_updateMarkerStrainPressure(self.h, dt)

    def updateGlobalStrainRateResidual(self, it=0):
        return self.L.ref_updateGlobalStrainRateResidual(self.h, it)

    def subgridStressChanges(self, dt, D):
        return self.L.ref_subgridStressChanges(self.h, dt, D)

    def updateMarkerStress(self):
        return self.L.ref_updateMarkerStress(self.h)

    def subgridTemperatureChanges(self, dt):
        return self.L.ref_subgridTemperatureChanges(self.h, dt)

    def advectMarkersRK(self, dt):
        return self.L.ref_advectMarkersRK(self.h, dt)


def goldsby_kohlstedt(s, T, d, P):
    """Vectorised viscosity.c:106-179 (returns effective viscosity)."""
    s, T, d, P = (np.ascontiguousarray(np.broadcast_to(a, np.broadcast(s, T, d, P).shape), dtype=np.float64).ravel()
                  for a in (s, T, d, P))
    out = np.empty_like(s)
    lib().ref_goldsbyKohlstedt_many(_dp(s), _dp(T), _dp(d), _dp(P), _dp(out), len(s))
    return out
