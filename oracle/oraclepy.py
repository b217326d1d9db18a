"""ctypes driver for oracle/liboracle.so, the CPU restatement of the marker path.

TEST INFRASTRUCTURE ONLY (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline
leg).  The interface mirrors oracle/refpy.RefProblem so that a test can run the
same sequence through the reference build and through the restatement."""
import ctypes
import os

import numpy as np

from fvmic2d_gb300.mic_types import NF, MARKER_DTYPE, MARKER_F64_OFFSETS
from . import build as _build

_lib = None
_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_I64P = ctypes.POINTER(ctypes.c_int64)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_build.build_oracle())
        sig = {
            "orc_create": (_P, [_I, _I, _D, _D, _DP, _DP]),
            "orc_destroy": (None, [_P]),
            "orc_get_grid": (None, [_P, _DP, _DP]),
            "orc_set_materials": (None, [_P, _P]),
            "orc_set_options": (None, [_P, _P]),
            "orc_set_jaumann": (None, [_P, _I]),
            "orc_set_bcs": (_I, [_P, _P]),
            "orc_set_nodal": (_I, [_P, _I, _DP]),
            "orc_get_nodal": (_I, [_P, _I, _DP]),
            "orc_find_marker_cells": (_I64, [_P, _P, _I64, _IP]),
            "orc_update_marker_rho": (None, [_P, _P, _I64]),
            "orc_max_marker_T": (_D, [_P, _P, _I64]),
            "orc_max_abs_sxx": (_D, [_P, _P, _I64]),
            "orc_project_marker_field": (_I, [_P, _P, _I64, _I, _DP, _I, _I, _I, _I]),
            "orc_project_markers_nodes_all2": (_I, [_P, _P, _I64]),
            "orc_project_nodal_to_markers": (_I, [_P, _P, _I64, _I, _I]),
            "orc_check_plastic_yielding": (_I, [_P, _P, _I64, _D, _IP]),
            "orc_limit_viscosity": (None, [_P, _P, _I64]),
            "orc_update_marker_strain_pressure": (_I, [_P, _P, _I64, _D]),
            "orc_update_global_strain_rate_residual": (_D, [_P, _P, _I64, _I]),
            "orc_subgrid_stress_changes": (_I, [_P, _P, _I64, _D, _D]),
            "orc_update_marker_stress": (_I, [_P, _P, _I64, _I64P]),
            "orc_subgrid_temperature_changes": (_I, [_P, _P, _I64, _D]),
            "orc_advect_markers_rk": (_I, [_P, _P, _I64, _D]),
            "orc_step": (_I, [_P, _P, _I64, _D, _D, _I, _DP]),
            "orc_gk_viscosity": (_D, [_D, _D, _D, _D]),
            "orc_sizeof": (_I64, [_I]),
            "orc_set_grain": (None, [_P, _DP, _I64]),
            "orc_gk_strain_rate": (_D, [_D, _D, _D, _D]),
            "orc_creep_stress": (_I, [_D, _D, _D, _D, _D, _DP, _IP]),
            "orc_creep_stress_batch": (_I, [_DP, _DP, _DP, _DP, _I64, _D, _DP, _P]),
            "orc_reset_markers": (None, [_P, _I64]),
            "orc_srand48_state": (ctypes.c_uint64, [ctypes.c_long]),
            "orc_nodal_stress_strain": (None, [_P, _D]),
            "orc_project_from_scalar": (_I, [_P, _P, _I64, _DP, _I]),
            "orc_save_markers_binary": (_I, [ctypes.c_char_p, _P, _I64, _D]),
            "orc_restart_from_markers": (_I64, [_P, ctypes.c_char_p, _P, _I64, _DP]),
            "orc_limit_displacement_timestep": (_D, [_P, _D, _D]),
            "orc_retrieve_solutions": (None, [_P, _DP, _D]),
            "orc_check_marker_density": (_I64, [_P, _P, _I64, _I64, _P, ctypes.POINTER(ctypes.c_uint64), _I64P,
                                                 _I64P]),
            "orc_distribute_uniform": (_I64, [_P, _P, _I64, _I, _I, ctypes.c_ulong]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_DP)


class OracleProblem:
    """Same surface as refpy.RefProblem, backed by the C restatement."""

    def __init__(self, wl, markers=None, jaumann=False):
        """jaumann: the stress rotation of the reference built with -DJAUMANN"""
        L = lib()
        g = wl.grid
        self.wl = wl
        self.NX, self.NY = g.NX, g.NY
        self.h = L.orc_create(g.NX, g.NY, g.LX, g.LY, _dp(g.x), _dp(g.y))
        self.materials, self.options, self.bcs = wl.materials, wl.options, wl.bcs
        L.orc_set_materials(self.h, ctypes.byref(self.materials))
        L.orc_set_options(self.h, ctypes.byref(self.options))
        L.orc_set_jaumann(self.h, 1 if jaumann else 0)
        if L.orc_set_bcs(self.h, ctypes.byref(self.bcs)) != 0:
            raise ValueError("boundary types other than 0/1 on the top-vx / left-vy walls are not supported")
        self.markers = np.array(wl.markers if markers is None else markers, dtype=MARKER_DTYPE, copy=True)
        for name, arr in wl.nodal.items():
            self.set_nodal(name, arr)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def _m(self):
        return self.markers.ctypes.data

    @property
    def n(self):
        return len(self.markers)

    def distribute_uniform(self, NMX, NMY, seed=0, cap=None):
        """resetMarkers + distributeMarkersUniformInDomain into a fresh array of capacity cap."""
        L = lib()
        cap = cap or NMX * NMY * (self.NX - 1) * (self.NY - 1) + 16
        mk = np.zeros(cap, dtype=MARKER_DTYPE)
        L.orc_reset_markers(mk.ctypes.data, cap)
        n = L.orc_distribute_uniform(self.h, mk.ctypes.data, cap, NMX, NMY, seed)
        if n < 0:
            raise ValueError("capacity exceeded")
        self.markers = mk[:n].copy()
        return mk, n

    def saveMarkersBinary(self, path, elapsed_time):
        if lib().orc_save_markers_binary(os.fsencode(path), self.markers.ctypes.data, len(self.markers),
                                         elapsed_time):
            raise IOError(path)

    def restartFromMarkers(self, path, cap):
        mk = np.zeros(cap, dtype=MARKER_DTYPE)
        t = ctypes.c_double(0.0)
        n = lib().orc_restart_from_markers(self.h, os.fsencode(path), mk.ctypes.data, cap, ctypes.byref(t))
        if n < 0:
            raise IOError(path)
        self.markers = mk[:n].copy()
        return t.value

    def projectMarkersNodesFromScalar(self, values, nodal):
        v = np.ascontiguousarray(values, dtype=np.float64)
        return lib().orc_project_from_scalar(self.h, self._m, self.n, _dp(v), NF[nodal])

    def nodalStressStrain(self, dt, gy=0.0):
        lib().orc_nodal_stress_strain(self.h, dt)

    def limitDisplacementTimestep(self, dt, factor):
        return lib().orc_limit_displacement_timestep(self.h, dt, factor)

    def retrieveSolutions(self, S, Kcont):
        S = np.ascontiguousarray(S, dtype=np.float64)
        lib().orc_retrieve_solutions(self.h, _dp(S), Kcont)

    def checkMarkerDensity(self, dopt, cap, state=None, seed=1):
        """checkMarkerDensity on a copy of the markers grown to capacity cap; returns
        (markers[:n_new], n_added, n_removed, rng state after)."""
        L = lib()
        mk = np.zeros(cap, dtype=MARKER_DTYPE)
        mk[:len(self.markers)] = self.markers
        st = ctypes.c_uint64(L.orc_srand48_state(seed) if state is None else state)
        na, nr = ctypes.c_int64(0), ctypes.c_int64(0)
        n = L.orc_check_marker_density(self.h, mk.ctypes.data, len(self.markers), cap, ctypes.byref(dopt),
                                       ctypes.byref(st), ctypes.byref(na), ctypes.byref(nr))
        if n < 0:
            raise RuntimeError("orc_check_marker_density failed with %d" % n)
        self.markers = mk[:n].copy()
        return self.markers, na.value, nr.value, st.value

    def grid_centres(self):
        xc = np.empty(self.NX + 1)
        yc = np.empty(self.NY + 1)
        lib().orc_get_grid(self.h, _dp(xc), _dp(yc))
        return xc, yc

    def set_nodal(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.NY, self.NX)
        assert lib().orc_set_nodal(self.h, NF[name], _dp(a)) == 0

    def get_nodal(self, name):
        a = np.empty((self.NY, self.NX))
        assert lib().orc_get_nodal(self.h, NF[name], _dp(a)) == 0
        return a

    def set_grain_size(self, d):
        self._grain = np.ascontiguousarray(d, dtype=np.float64)
        lib().orc_set_grain(self.h, _dp(self._grain), len(self._grain))

    def findMarkerCells(self):
        err = ctypes.c_int(0)
        nout = lib().orc_find_marker_cells(self.h, self._m, self.n, ctypes.byref(err))
        if err.value:
            raise RuntimeError("impossible cell index")
        return nout

    def updateMarkerRho(self):
        lib().orc_update_marker_rho(self.h, self._m, self.n)

    def maxMarkerT(self):
        return lib().orc_max_marker_T(self.h, self._m, self.n)

    def maxAbsSxx(self):
        return lib().orc_max_abs_sxx(self.h, self._m, self.n)

    def projectMarkersNodesAll2(self):
        return lib().orc_project_markers_nodes_all2(self.h, self._m, self.n)

    def projectMarkerFieldToNodes(self, field, out, stagx, stagy, method, matprop=None):
        off = -1 if field is None else MARKER_F64_OFFSETS[field]
        mp = None
        if matprop is not None:
            self._mp = np.ascontiguousarray(matprop, dtype=np.float64)
            mp = _dp(self._mp)
        return lib().orc_project_marker_field(self.h, self._m, self.n, off, mp, NF[out], stagx, stagy, method)

    def projectNodalFieldToMarkersS(self, nodal, field):
        return lib().orc_project_nodal_to_markers(self.h, self._m, self.n, NF[nodal], MARKER_F64_OFFSETS[field])

    def checkPlasticYielding(self, dt, t=0.0):
        y = ctypes.c_int(0)
        e = lib().orc_check_plastic_yielding(self.h, self._m, self.n, dt, ctypes.byref(y))
        if e:
            raise RuntimeError("viscosity law undefined")
        return y.value

    def limitViscosity(self):
        lib().orc_limit_viscosity(self.h, self._m, self.n)

    def updateMarkerStrainPressure(self, dt):
        return lib().orc_update_marker_strain_pressure(self.h, self._m, self.n, dt)

    def updateGlobalStrainRateResidual(self, it=0):
        return lib().orc_update_global_strain_rate_residual(self.h, self._m, self.n, it)

    def subgridStressChanges(self, dt, D):
        return lib().orc_subgrid_stress_changes(self.h, self._m, self.n, dt, D)

    def updateMarkerStress(self):
        return lib().orc_update_marker_stress(self.h, self._m, self.n, None)

    def subgridTemperatureChanges(self, dt):
        return lib().orc_subgrid_temperature_changes(self.h, self._m, self.n, dt)

    def advectMarkersRK(self, dt):
        return lib().orc_advect_markers_rk(self.h, self._m, self.n, dt)

    def step(self, dt_disp, dt_thermal, subgrid_stress=True):
        r = ctypes.c_double(0.0)
        e = lib().orc_step(self.h, self._m, self.n, dt_disp, dt_thermal, int(subgrid_stress), ctypes.byref(r))
        return e, r.value


def gk_viscosity(s, T, d, P):
    f = lib().orc_gk_viscosity
    return np.array([f(float(a), float(b), float(c), float(e)) for a, b, c, e in
                     np.broadcast(np.asarray(s), np.asarray(T), np.asarray(d), np.asarray(P))])


def gk_strain_rate(s, T, d, P):
    """Strain rate of the reference law at stress s (viscosity.c:106-179, s / (2 eta))."""
    f = lib().orc_gk_strain_rate
    return np.array([f(float(a), float(b), float(c), float(e)) for a, b, c, e in
                     np.broadcast(np.asarray(s), np.asarray(T), np.asarray(d), np.asarray(P))])


def creep_stress(edot, T, d, P, rtol=1e-14):
    """Stress at which the reference law's strain rate equals edot (oracle solve, one C call)."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in np.broadcast_arrays(edot, T, d, P)]
    n = len(arrs[0])
    out = np.zeros(n)
    its = np.zeros(n, dtype=np.int32)
    lib().orc_creep_stress_batch(*[_dp(a) for a in arrs], n, rtol, _dp(out), its.ctypes.data)
    return out, its
