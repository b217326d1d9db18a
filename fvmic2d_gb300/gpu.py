"""Python host side of the GB300 marker path: ctypes over the C ABI of libmic_gb300.so.

``MicProblem`` mirrors fvmic2d's entry points (findMarkerCells,
projectMarkersNodesAll2, checkPlasticYielding, ...) with the reference's argument
meaning, so a test can drive the same sequence through the reference build, the CPU
oracle and the GPU.  There is no CPU fallback: a missing library or GPU raises.
"""
import ctypes
import os

import numpy as np

from .mic_types import MARKER_DTYPE, MARKER_F64_OFFSETS, NF

HERE = os.path.dirname(os.path.abspath(__file__))

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_I64 = ctypes.c_int64
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_I64P = ctypes.POINTER(ctypes.c_int64)

SIGNATURES = {
    "mic_version": (_I, []),
    "mic_error_string": (ctypes.c_char_p, [_I]),
    "mic_create": (_I, [ctypes.POINTER(_P), _I, _P, _I, _I, _D, _D, _DP, _DP, _I64]),
    "mic_destroy": (_I, [_P]),
    "mic_set_materials": (_I, [_P, _P]),
    "mic_set_options": (_I, [_P, _P]),
    "mic_set_bcs": (_I, [_P, _P]),
    "mic_get_bcs": (_I, [_P, _P]),
    "mic_set_stress_rotation": (_I, [_P, _I]),
    "mic_get_stress_rotation": (_I, [_P, _IP]),
    "mic_get_grid_centres": (_I, [_P, _DP, _DP]),
    "mic_markers_upload": (_I, [_P, _P, _I64]),
    "mic_markers_download": (_I, [_P, _P, _I64]),
    "mic_markers_count": (_I, [_P, _I64P]),
    "mic_nodal_upload": (_I, [_P, _I, _DP]),
    "mic_nodal_upload_many": (_I, [_P, _IP, _P, _I]),
    "mic_nodal_download_many": (_I, [_P, _IP, _P, _I]),
    "mic_nodal_download": (_I, [_P, _I, _DP]),
    "mic_nodal_device_ptr": (_I, [_P, _I, ctypes.POINTER(_DP)]),
    "mic_find_marker_cells": (_I, [_P, _I64P]),
    "mic_update_marker_rho": (_I, [_P]),
    "mic_max_marker_T": (_I, [_P, _DP]),
    "mic_project_markers_nodes_all2": (_I, [_P]),
    "mic_project_marker_field_to_nodes": (_I, [_P, _I, _DP, _I, _I, _I, _I]),
    "mic_project_nodal_field_to_markers": (_I, [_P, _I, _I]),
    "mic_check_plastic_yielding": (_I, [_P, _D, _IP, _D]),
    "mic_update_viscosity": (_I, [_P]),
    "mic_limit_viscosity": (_I, [_P]),
    "mic_update_marker_strain_pressure": (_I, [_P, _D]),
    "mic_update_global_strain_rate_residual": (_I, [_P, _I, _DP]),
    "mic_check_convergence": (_I, [_P, _D, _D, _I, _IP]),
    "mic_subgrid_stress_changes": (_I, [_P, _D, _D]),
    "mic_update_marker_stress": (_I, [_P]),
    "mic_subgrid_temperature_changes": (_I, [_P, _D]),
    "mic_advect_markers_rk": (_I, [_P, _D]),
    "mic_max_abs_sxx": (_I, [_P, _DP]),
    "mic_step_pre_stokes": (_I, [_P, _D, _IP, _DP]),
    "mic_step_post_stokes": (_I, [_P, _D, _I, _DP]),
    "mic_step_post_thermal": (_I, [_P, _D, _DP]),
    "mic_step": (_I, [_P, _D, _D, _I, _DP]),
    "mic_synchronize": (_I, [_P]),
    "mic_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "mic_get_status": (_I, [_P, _P]),
    "mic_debug_sorted_ids": (_I, [_P, _P]),
    "mic_debug_cell_start": (_I, [_P, _P]),
    "mic_debug_div_sp": (_I, [_P, _P, _P, _I64, _P]),
    "mic_markers_reset_host": (_I, [_P, _I64]),
    "mic_get_strain_rate_residual": (_I, [_P, _I, _DP]),
    "mic_set_strain_rate_residual": (_I, [_P, _I, _D]),
    "mic_launch_count": (_I, [_P, _I64P]),
    "mic_profile_enable": (_I, [_P, _I]),
    "mic_profile_read": (_I, [_P, _I, _P, _DP, _I64P, _IP]),
    "mic_autotune": (_I, [_P, _D, _D, _I, _I, _IP]),
    "mic_get_tuning": (_I, [_P, _IP, _I]),
    "mic_set_tuning": (_I, [_P, _IP, _I]),
    "mic_bin_sort_noalloc": (_I, [_P, _P, _I64, _P, _P, _I, _I, _D, _D, _P, _P, _P, _P, _P, _I64P]),
    "mic_creep_configure": (_I, [_P, _I, _D, _I, _I, _D]),
    "mic_markers_set_grain_size": (_I, [_P, _DP, _I64]),
    "mic_creep_param_count": (_I, []),
    "mic_creep_set_mlp": (_I, [_P, _P, _I]),
    "mic_creep_get_mlp": (_I, [_P, _P, _I]),
    "mic_creep_train": (_I, [_P, _I64, _I, _I, ctypes.c_float, ctypes.c_uint64, _P]),
    "mic_creep_mlp_grad": (_I, [_P, _P, _P, _P, _I, _P, _P]),
    "mic_creep_solve_batch": (_I, [_P, _DP, _DP, _DP, _DP, _I64, _I, _DP, _P, _DP, _P]),
    "mic_creep_mlp_infer": (_I, [_P, _P, _I64, _I, _P]),
    "mic_creep_stats": (_I, [_P, _I64P, _I64P, _I64P, _DP, _I64P]),
    "mic_creep_set_tc_wait_limit": (_I, [_P, _I]),
    "mic_creep_tc_stats": (_I, [_P, _I64P, _I64P]),
    "mic_reset_markers": (_I, [_P]),
    "mic_marker_count": (_I, [_P, _I64P]),
    "mic_distribute_markers_uniform_in_domain": (_I, [_P, _I, _I, ctypes.c_ulong, _I64P]),
    "mic_markers_fill": (_I, [_P, _I, _D]),
    "mic_ensemble_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(_P), _I]),
    "mic_ensemble_destroy": (_I, [_P]),
    "mic_ensemble_step": (_I, [_P, _DP, _DP, _I, _I]),
    "mic_ensemble_autotune": (_I, [_P, _DP, _DP, _I, _I, _IP]),
    "mic_ensemble_synchronize": (_I, [_P]),
    "mic_ensemble_launch_count": (_I, [_P, _I64P, _I64P]),
    "mic_ensemble_get_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "mic_ensemble_set_schedule": (_I, [_P, _I, _I, _I, _I]),
    "mic_ensemble_get_schedule": (_I, [_P, _IP, _IP, _IP, _IP]),
    "mic_check_marker_density": (_I, [_P, _P, _I64P, _I64P]),
    "mic_nodal_stress_strain": (_I, [_P, _D, _D]),
    "mic_project_markers_nodes_from_scalar": (_I, [_P, _DP, _I]),
    "mic_creep_newton": (_I, [_P, _DP, _DP, _DP, _DP, _I64, _DP, _P, _DP]),
    "mic_surrogate_train": (_I, [_P, _I64, _I, _I, ctypes.c_float, ctypes.c_uint64, _P]),
    "mic_surrogate_infer": (_I, [_P, _P, _I64, _I, _P]),
    "mic_save_markers_binary": (_I, [_P, ctypes.c_char_p, _D]),
    "mic_restart_from_markers": (_I, [_P, ctypes.c_char_p, _DP]),
    "mic_limit_displacement_timestep": (_I, [_P, _D, _DP]),
    "mic_retrieve_solutions": (_I, [_P, _DP, _D, _IP]),
    "mic_density_seed": (_I, [_P, ctypes.c_long]),
    "mic_density_rng_state": (_I, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "mic_density_fill_rounds": (_I, [_P, _IP]),
    "mic_form_vep_system": (_I, [_P, _P, _D, _DP, _DP]),
    "mic_enforce_thermal_bcs": (_I, [_P, _P]),
    "mic_form_thermal_system": (_I, [_P, _P, _D, _I]),
    "mic_system_size": (_I, [_P, _I, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "mic_system_get": (_I, [_P, _I, _P, _P, _DP, _DP]),
    "mic_linear_solve": (_I, [_P, _I]),
    "mic_solution_get": (_I, [_P, _I, _DP]),
    "mic_system_band": (_I, [_P, _I, _IP, _IP]),
    "mic_subduction_timestep": (_I, [_P, _P, _D, _P]),
    "mic_adiabatic_heating": (_I, [_P, _D]),
    "mic_reset_nodal_fields": (_I, [_P]),
    "mic_initial_conditions_van_keken": (_I, [_P, _P]),
    "mic_nusselt_number": (_I, [_P, _D, _D, _DP]),
    "mic_rms_velocity": (_I, [_P, _DP]),
    "mic_subduction_timestep_many": (_I, [_P, _I, _P, _DP, _P, _IP, _I]),
    "mic_host_alloc": (_I, [ctypes.POINTER(_P), _I64]),
    "mic_host_free": (_I, [_P]),
}

_libs = {}

NOALLOC_MAX_MARKERS = 1048576  # MIC_NOALLOC_MAX_MARKERS
NOALLOC_MAX_CELLS = 1048576    # MIC_NOALLOC_MAX_CELLS
MIC_ROTATION_EXACT, MIC_ROTATION_JAUMANN = 0, 1  # mic_set_stress_rotation


class MicError(RuntimeError):
    def __init__(self, code, what):
        self.code = code
        super().__init__("%s failed: %s (code %d)" % (what, load().mic_error_string(code).decode(), code))


def library_path(exact=False):
    return os.path.join(HERE, "libmic_gb300_exact.so" if exact else "libmic_gb300.so")


def load(exact=False):
    """Load the CUDA library; raises if it was not built (there is no fallback)."""
    key = bool(exact)
    if key not in _libs:
        path = library_path(exact)
        if not os.path.exists(path):
            raise RuntimeError("%s is missing: run __graft_entry__.build() (nvcc, sm_103a)" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _libs[key] = L
    return _libs[key]


class Status(ctypes.Structure):
    _fields_ = [("bad_cell", ctypes.c_uint64), ("nan_residual", ctypes.c_uint64), ("nan_dsxy", ctypes.c_uint64),
                ("bad_law", ctypes.c_uint64), ("n_out", ctypes.c_uint64), ("is_yielding", ctypes.c_int32)]


def _dp(a):
    return a.ctypes.data_as(_DP)


# kernels whose launch block size mic_autotune picks, in the library's MIC_TUNE_* order
TUNE_KERNELS = ["k_advect", "k_strain_pressure", "k_yield", "k_subgrid_stress_markers", "k_update_marker_stress",
                "k_subgridT_markers", "k_subgridT_apply", "k_reorder", "k_find_cells", "k_update_rho"]


class MicProblem:
    """A device context holding one grid, its nodal fields and a marker set."""

    def __init__(self, wl, markers=None, exact=False, device=0, capacity=None, stream=None, jaumann=False):
        """jaumann: advectMarkersRK's stress rotation as the reference built with -DJAUMANN"""
        self.L = L = load(exact)
        g = wl.grid
        self.wl = wl
        self.NX, self.NY = g.NX, g.NY
        mk = wl.markers if markers is None else markers
        cap = len(mk) if capacity is None else capacity
        h = _P()
        self._check(L.mic_create(ctypes.byref(h), device, stream, g.NX, g.NY, g.LX, g.LY, _dp(g.x), _dp(g.y), cap),
                    "mic_create")
        self.h = h
        self.materials, self.options, self.bcs = wl.materials, wl.options, wl.bcs
        self._check(L.mic_set_materials(self.h, ctypes.byref(self.materials)), "mic_set_materials")
        self._check(L.mic_set_options(self.h, ctypes.byref(self.options)), "mic_set_options")
        self._check(L.mic_set_bcs(self.h, ctypes.byref(self.bcs)), "mic_set_bcs")
        if jaumann:
            self.set_stress_rotation(MIC_ROTATION_JAUMANN)
        self.upload_markers(mk)
        for name, arr in wl.nodal.items():
            self.set_nodal(name, arr)

    def _check(self, code, what):
        if code != 0:
            raise MicError(code, what)

    def set_stress_rotation(self, rotation):
        """MIC_ROTATION_EXACT (markers.c:2158-2164) or MIC_ROTATION_JAUMANN (2147-2156)"""
        self._check(self.L.mic_set_stress_rotation(self.h, rotation), "mic_set_stress_rotation")

    def stress_rotation(self):
        r = ctypes.c_int(-1)
        self._check(self.L.mic_get_stress_rotation(self.h, ctypes.byref(r)), "mic_get_stress_rotation")
        return r.value

    def close(self):
        if getattr(self, "h", None):
            self.L.mic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- marker lifecycle (markers.c:255-400) ---------------------------------
    def resetMarkers(self):
        self._check(self.L.mic_reset_markers(self.h), "mic_reset_markers")

    def distributeMarkersUniformInDomain(self, NMX, NMY, seed=0):
        n = ctypes.c_int64(0)
        self._check(self.L.mic_distribute_markers_uniform_in_domain(self.h, NMX, NMY, seed, ctypes.byref(n)),
                    "mic_distribute_markers_uniform_in_domain")
        self.n = n.value
        return self.n

    def projectMarkersNodesFromScalar(self, values, nodal):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.L.mic_project_markers_nodes_from_scalar(self.h, _dp(v), NF[nodal]),
                    "mic_project_markers_nodes_from_scalar")
        return 0

    def saveMarkersBinary(self, path, elapsed_time):
        self._check(self.L.mic_save_markers_binary(self.h, os.fsencode(path), elapsed_time), "mic_save_markers_binary")

    def restartFromMarkers(self, path):
        t = ctypes.c_double(0.0)
        self._check(self.L.mic_restart_from_markers(self.h, os.fsencode(path), ctypes.byref(t)),
                    "mic_restart_from_markers")
        self.n = self._count()
        return t.value

    def nodalStressStrain(self, dt, gy=0.0):
        self._check(self.L.mic_nodal_stress_strain(self.h, dt, gy), "mic_nodal_stress_strain")

    def limitDisplacementTimestep(self, dt, factor):
        d = ctypes.c_double(dt)
        self._check(self.L.mic_limit_displacement_timestep(self.h, factor, ctypes.byref(d)),
                    "mic_limit_displacement_timestep")
        return d.value

    def retrieveSolutions(self, S, Kcont):
        """S: the solver's vector (host), or None for the solution mic_linear_solve left on the
        device"""
        nan = ctypes.c_int(0)
        if S is None:
            self._check(self.L.mic_retrieve_solutions(self.h, None, Kcont, ctypes.byref(nan)),
                        "mic_retrieve_solutions")
            return nan.value
        S = np.ascontiguousarray(S, dtype=np.float64)
        self._check(self.L.mic_retrieve_solutions(self.h, _dp(S), Kcont, ctypes.byref(nan)), "mic_retrieve_solutions")
        return nan.value

    STOKES, THERMAL = 0, 1

    def formVEPSystem(self, sopt, dt):
        """formVEPSystem (vep_system.c:12) on the device; returns (Kbond, Kcont)"""
        kb, kc = ctypes.c_double(0.0), ctypes.c_double(0.0)
        self._check(self.L.mic_form_vep_system(self.h, ctypes.byref(sopt), dt, ctypes.byref(kb), ctypes.byref(kc)),
                    "mic_form_vep_system")
        return kb.value, kc.value

    def enforceThermalBCs1(self, sopt):
        self._check(self.L.mic_enforce_thermal_bcs(self.h, ctypes.byref(sopt)), "mic_enforce_thermal_bcs")

    def formThermalSystem(self, sopt, dt, doSteady=0):
        self._check(self.L.mic_form_thermal_system(self.h, ctypes.byref(sopt), dt, doSteady),
                    "mic_form_thermal_system")

    def system(self, which):
        """the assembled system as (rowptr, cols, vals, rhs), columns ascending"""
        nr, nnz = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.L.mic_system_size(self.h, which, ctypes.byref(nr), ctypes.byref(nnz)), "mic_system_size")
        rp = np.zeros(nr.value + 1, dtype=np.int32)
        c = np.zeros(max(nnz.value, 1), dtype=np.int32)
        v = np.zeros(max(nnz.value, 1))
        rhs = np.zeros(nr.value)
        self._check(self.L.mic_system_get(self.h, which, rp.ctypes.data, c.ctypes.data, _dp(v), _dp(rhs)),
                    "mic_system_get")
        return rp, c[:nnz.value], v[:nnz.value], rhs

    def linear_solve(self, which):
        """direct solve of an assembled system on the device (kspLinearSolve, preonly + LU)"""
        self._check(self.L.mic_linear_solve(self.h, which), "mic_linear_solve")

    def solution(self, which):
        nn = self.NX * self.NY
        out = np.zeros(3 * nn if which == self.STOKES else nn)
        self._check(self.L.mic_solution_get(self.h, which, _dp(out)), "mic_solution_get")
        return out

    def adiabaticHeating(self, gy):
        """adiabaticHeating (adiabaticHeating.c:7) added to the heating field (main:377)"""
        self._check(self.L.mic_adiabatic_heating(self.h, gy), "mic_adiabatic_heating")

    def get_bcs(self):
        """the context's boundary conditions (mic_bcs)"""
        from .mic_types import BCs

        b = BCs()
        self._check(self.L.mic_get_bcs(self.h, ctypes.byref(b)), "mic_get_bcs")
        return b

    def resetNodalFields(self):
        self._check(self.L.mic_reset_nodal_fields(self.h), "mic_reset_nodal_fields")

    def initialConditionsVanKeken(self, sopt):
        """initialConditionsVanKeken (benchmarkInitialConditions.c:8) on the device; the left and
        top boundary conditions change as the reference changes them"""
        self._check(self.L.mic_initial_conditions_van_keken(self.h, ctypes.byref(sopt)),
                    "mic_initial_conditions_van_keken")

    def nusseltNumber(self, bottom_T, top_T):
        v = ctypes.c_double(0.0)
        self._check(self.L.mic_nusselt_number(self.h, bottom_T, top_T, ctypes.byref(v)), "mic_nusselt_number")
        return v.value

    def rmsVelocity(self):
        v = ctypes.c_double(0.0)
        self._check(self.L.mic_rms_velocity(self.h, ctypes.byref(v)), "mic_rms_velocity")
        return v.value

    def subductionTimestep(self, topt, elapsed_time=0.0):
        """one time step of main_subduction.c on the device; returns the report as a dict"""
        from .mic_types import TimestepReport

        rep = TimestepReport()
        self._check(self.L.mic_subduction_timestep(self.h, ctypes.byref(topt), elapsed_time, ctypes.byref(rep)),
                    "mic_subduction_timestep")
        self.n = self._count()
        return rep.as_dict()

    def system_band(self, which):
        kl, ku = ctypes.c_int(0), ctypes.c_int(0)
        self._check(self.L.mic_system_band(self.h, which, ctypes.byref(kl), ctypes.byref(ku)), "mic_system_band")
        return kl.value, ku.value

    def checkMarkerDensity(self, dopt):
        """markers.c:455-781 on the device; returns (n_added, n_removed)."""
        a, r = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.L.mic_check_marker_density(self.h, ctypes.byref(dopt), ctypes.byref(a), ctypes.byref(r)),
                    "mic_check_marker_density")
        self.n = self._count()
        return a.value, r.value

    def _count(self):
        n = ctypes.c_int64(0)
        self._check(self.L.mic_marker_count(self.h, ctypes.byref(n)), "mic_marker_count")
        return n.value

    def density_seed(self, seed):
        self._check(self.L.mic_density_seed(self.h, seed), "mic_density_seed")

    def density_state(self):
        v = ctypes.c_uint64(0)
        self._check(self.L.mic_density_rng_state(self.h, ctypes.byref(v), None), "mic_density_rng_state")
        return v.value

    def density_fill_rounds(self):
        """rounds the last checkMarkerDensity took to settle the copies (negative: in-order fill)"""
        v = ctypes.c_int(0)
        self._check(self.L.mic_density_fill_rounds(self.h, ctypes.byref(v)), "mic_density_fill_rounds")
        return v.value

    def fill(self, field, value):
        """Set one marker field (a MARKER_DTYPE name) to value on every marker."""
        off = MARKER_DTYPE.fields[field][1]
        self._check(self.L.mic_markers_fill(self.h, off, float(value)), "mic_markers_fill")

    # ---- transfers -----------------------------------------------------------
    def upload_markers(self, mk):
        mk = np.ascontiguousarray(mk, dtype=MARKER_DTYPE)
        self.n = len(mk)
        self._check(self.L.mic_markers_upload(self.h, mk.ctypes.data, self.n), "mic_markers_upload")

    @property
    def markers(self):
        out = np.zeros(self.n, dtype=MARKER_DTYPE)
        self._check(self.L.mic_markers_download(self.h, out.ctypes.data, self.n), "mic_markers_download")
        return out

    def set_nodal(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.NY, self.NX)
        self._check(self.L.mic_nodal_upload(self.h, NF[name], _dp(a)), "mic_nodal_upload")

    def get_nodal(self, name):
        a = np.empty((self.NY, self.NX))
        self._check(self.L.mic_nodal_download(self.h, NF[name], _dp(a)), "mic_nodal_download")
        return a

    def grid_centres(self):
        xc = np.empty(self.NX + 1)
        yc = np.empty(self.NY + 1)
        self._check(self.L.mic_get_grid_centres(self.h, _dp(xc), _dp(yc)), "mic_get_grid_centres")
        return xc, yc

    def status(self):
        s = Status()
        self._check(self.L.mic_get_status(self.h, ctypes.byref(s)), "mic_get_status")
        return s

    def sorted_ids(self):
        ids = np.empty(self.n, dtype=np.int32)
        self._check(self.L.mic_debug_sorted_ids(self.h, ids.ctypes.data), "mic_debug_sorted_ids")
        return ids

    def cell_start(self):
        cs = np.empty((self.NX - 1) * (self.NY - 1) + 2, dtype=np.int32)
        self._check(self.L.mic_debug_cell_start(self.h, cs.ctypes.data), "mic_debug_cell_start")
        return cs

    def debug_div_sp(self, num, den):
        """num / den by the kernels' grid-spacing division (mic_debug_div_sp)"""
        num = np.ascontiguousarray(num, dtype=np.float64)
        den = np.ascontiguousarray(den, dtype=np.float64)
        q = np.zeros(len(num))
        self._check(self.L.mic_debug_div_sp(self.h, num.ctypes.data, den.ctypes.data, len(num), q.ctypes.data),
                    "mic_debug_div_sp")
        return q

    def launch_count(self):
        n = ctypes.c_int64(0)
        self._check(self.L.mic_launch_count(self.h, ctypes.byref(n)), "mic_launch_count")
        return n.value

    def autotune(self, dt_disp, dt_thermal, subgrid_stress=1, steps=2):
        """mic_autotune: per-kernel block sizes measured on this workload; state left unchanged.
        Returns {kernel: block size}."""
        out = (ctypes.c_int * len(TUNE_KERNELS))()
        self._check(self.L.mic_autotune(self.h, dt_disp, dt_thermal, int(subgrid_stress), steps, out),
                    "mic_autotune")
        return dict(zip(TUNE_KERNELS, list(out)))

    def tuning(self):
        out = (ctypes.c_int * len(TUNE_KERNELS))()
        self._check(self.L.mic_get_tuning(self.h, out, len(TUNE_KERNELS)), "mic_get_tuning")
        return dict(zip(TUNE_KERNELS, list(out)))

    def set_tuning(self, blocks):
        """blocks: {kernel: size} (sizes 0, 128, 256 or 512; 0 = default) or a list in kernel order"""
        vals = [int(blocks.get(k, 0)) for k in TUNE_KERNELS] if isinstance(blocks, dict) else [int(b) for b in blocks]
        arr = (ctypes.c_int * len(vals))(*vals)
        self._check(self.L.mic_set_tuning(self.h, arr, len(vals)), "mic_set_tuning")

    def profile_enable(self, capacity):
        self._check(self.L.mic_profile_enable(self.h, capacity), "mic_profile_enable")

    def profile_read(self):
        """{kernel name: (total ms, launches)} over the records since profile_enable."""
        cap = 128
        names = ctypes.create_string_buffer(48 * cap)
        tot = np.zeros(cap)
        cnt = np.zeros(cap, dtype=np.int64)
        nk = ctypes.c_int(0)
        self._check(self.L.mic_profile_read(self.h, cap, names, _dp(tot), cnt.ctypes.data_as(_I64P),
                                             ctypes.byref(nk)), "mic_profile_read")
        out = {}
        for u in range(min(nk.value, cap)):
            nm = names.raw[48 * u: 48 * u + 48].split(b"\0", 1)[0].decode()
            out[nm] = (float(tot[u]), int(cnt[u]))
        return out

    # ---- composite creep closure (law 7) ----------------------------------------
    def set_grain_size(self, d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        self._check(self.L.mic_markers_set_grain_size(self.h, _dp(d), len(d)), "mic_markers_set_grain_size")

    def creep_configure(self, mode=0, tol=2e-14, maxit=60, polish_iters=3, polish_tol=1e-7):
        self._check(self.L.mic_creep_configure(self.h, mode, tol, maxit, polish_iters, polish_tol),
                    "mic_creep_configure")

    def creep_train(self, nsamples=1 << 21, batch=4096, steps=10000, lr=3e-3, seed=1):
        hist = np.zeros(steps, dtype=np.float32)
        self._check(self.L.mic_creep_train(self.h, nsamples, batch, steps, lr, seed, hist.ctypes.data),
                    "mic_creep_train")
        return hist

    def creep_params(self):
        n = self.L.mic_creep_param_count()
        p = np.zeros(n, dtype=np.float32)
        self._check(self.L.mic_creep_get_mlp(self.h, p.ctypes.data, n), "mic_creep_get_mlp")
        return p

    def creep_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.L.mic_creep_set_mlp(self.h, p.ctypes.data, len(p)), "mic_creep_set_mlp")

    def creep_grad(self, params, feats, targets):
        params = np.ascontiguousarray(params, dtype=np.float32)
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(len(params) - 2, dtype=np.float32)
        loss = ctypes.c_float(0.0)
        self._check(self.L.mic_creep_mlp_grad(self.h, params.ctypes.data, feats.ctypes.data, targets.ctypes.data,
                                              len(targets), g.ctypes.data, ctypes.byref(loss)), "mic_creep_mlp_grad")
        return g, loss.value

    def creep_solve(self, edot, T, d, P, mode=0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in np.broadcast_arrays(edot, T, d, P)]
        n = len(arrs[0])
        s = np.zeros(n)
        it = np.zeros(n, dtype=np.int32)
        res = np.zeros(n)
        fb = np.zeros(n, dtype=np.int32)
        self._check(self.L.mic_creep_solve_batch(self.h, *[_dp(a) for a in arrs], n, mode, _dp(s), it.ctypes.data,
                                                 _dp(res), fb.ctypes.data), "mic_creep_solve_batch")
        return s, it, res, fb

    def creep_infer(self, feat, mode):
        """Network outputs for normalised features (n x 4): mode 1 FP32 CUDA cores, 2 tensor cores."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        y = np.zeros(len(feat), dtype=np.float32)
        self._check(self.L.mic_creep_mlp_infer(self.h, feat.ctypes.data, len(feat), mode, y.ctypes.data),
                    "mic_creep_mlp_infer")
        return y

    def creep_stats(self):
        a, b, c, t = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        r = ctypes.c_double(0.0)
        self._check(self.L.mic_creep_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                           ctypes.byref(r), ctypes.byref(t)), "mic_creep_stats")
        return {"markers": a.value, "iterations": b.value, "fallbacks": c.value, "max_residual": r.value,
                "tc_timeouts": t.value}

    def creep_set_tc_wait_limit(self, rounds):
        """try_wait rounds on each tensor-core tile's completion before its block gives up"""
        self._check(self.L.mic_creep_set_tc_wait_limit(self.h, int(rounds)), "mic_creep_set_tc_wait_limit")

    def creep_tc_stats(self):
        t, d = ctypes.c_int64(0), ctypes.c_int64(0)
        self._check(self.L.mic_creep_tc_stats(self.h, ctypes.byref(t), ctypes.byref(d)), "mic_creep_tc_stats")
        return {"tile_timeouts": t.value, "drain_timeouts": d.value}

    def synchronize(self):
        self._check(self.L.mic_synchronize(self.h), "mic_synchronize")

    def stream(self):
        s = _P()
        self._check(self.L.mic_get_stream(self.h, ctypes.byref(s)), "mic_get_stream")
        return s.value

    # ---- fvmic2d entry points --------------------------------------------------
    def findMarkerCells(self):
        n = ctypes.c_int64(0)
        self._check(self.L.mic_find_marker_cells(self.h, ctypes.byref(n)), "findMarkerCells")
        return n.value

    def updateMarkerRho(self):
        self._check(self.L.mic_update_marker_rho(self.h), "updateMarkerRho")

    def maxMarkerT(self):
        v = ctypes.c_double(0.0)
        self._check(self.L.mic_max_marker_T(self.h, ctypes.byref(v)), "maxMarkerT")
        return v.value

    def maxAbsSxx(self):
        v = ctypes.c_double(0.0)
        self._check(self.L.mic_max_abs_sxx(self.h, ctypes.byref(v)), "maxAbsSxx")
        return v.value

    def projectMarkersNodesAll2(self):
        self._check(self.L.mic_project_markers_nodes_all2(self.h), "projectMarkersNodesAll2")
        return 0

    def projectMarkerFieldToNodes(self, field, out, stagx, stagy, method, matprop=None):
        off = -1 if field is None else MARKER_F64_OFFSETS[field]
        mp = None
        if matprop is not None:
            self._mp = np.zeros(8)
            self._mp[: len(matprop)] = matprop
            mp = _dp(self._mp)
        self._check(self.L.mic_project_marker_field_to_nodes(self.h, off, mp, NF[out], stagx, stagy, method),
                    "projectMarkerFieldToNodes")
        return 0

    def projectNodalFieldToMarkersS(self, nodal, field):
        self._check(self.L.mic_project_nodal_field_to_markers(self.h, NF[nodal], MARKER_F64_OFFSETS[field]),
                    "projectNodalFieldToMarkersS")
        return 0

    def checkPlasticYielding(self, dt, t=0.0):
        y = ctypes.c_int(0)
        self._check(self.L.mic_check_plastic_yielding(self.h, dt, ctypes.byref(y), t), "checkPlasticYielding")
        return y.value

    def updateViscosity(self):
        self._check(self.L.mic_update_viscosity(self.h), "updateViscosity")

    def limitViscosity(self):
        self._check(self.L.mic_limit_viscosity(self.h), "limitViscosity")

    def updateMarkerStrainPressure(self, dt):
        self._check(self.L.mic_update_marker_strain_pressure(self.h, dt), "updateMarkerStrainPressure")
        return 0

    def updateGlobalStrainRateResidual(self, it=0):
        r = ctypes.c_double(0.0)
        self._check(self.L.mic_update_global_strain_rate_residual(self.h, it, ctypes.byref(r)),
                    "updateGlobalStrainRateResidual")
        return r.value

    def checkConvergence(self, atol, rtol, it):
        c = ctypes.c_int(0)
        self._check(self.L.mic_check_convergence(self.h, atol, rtol, it, ctypes.byref(c)), "checkConvergence")
        return c.value

    def subgridStressChanges(self, dt, D):
        self._check(self.L.mic_subgrid_stress_changes(self.h, dt, D), "subgridStressChanges")
        return 0

    def updateMarkerStress(self):
        self._check(self.L.mic_update_marker_stress(self.h), "updateMarkerStress")
        return 0

    def subgridTemperatureChanges(self, dt):
        self._check(self.L.mic_subgrid_temperature_changes(self.h, dt), "subgridTemperatureChanges")
        return 0

    def advectMarkersRK(self, dt):
        self._check(self.L.mic_advect_markers_rk(self.h, dt), "advectMarkersRK")
        return 0

    def step(self, dt_disp, dt_thermal, subgrid_stress=True):
        r = ctypes.c_double(0.0)
        self._check(self.L.mic_step(self.h, dt_disp, dt_thermal, int(subgrid_stress), ctypes.byref(r)), "mic_step")
        return 0, r.value


def initialize_markers(P, NMX, NMY, seed=0, mat=0, T_field="lastT"):
    """The reference's marker set-up on the device (main_subduction.c:175-202): resetMarkers,
    distributeMarkersUniformInDomain, material id, cells, temperature from a nodal field
    (projectNodalFieldToMarkersS) and viscosity from it (updateViscosity)."""
    P.resetMarkers()
    n = P.distributeMarkersUniformInDomain(NMX, NMY, seed)
    P.fill("Mat", mat)
    P.findMarkerCells()
    P.projectNodalFieldToMarkersS(T_field, "T")
    P.updateViscosity()
    return n


class MicEnsemble:
    """Independent problems stepped together (mic_ensemble_*): members are MicProblem objects,
    each on its own context stream."""

    def __init__(self, members):
        self.members = list(members)
        self.L = self.members[0].L
        arr = (_P * len(self.members))(*[m.h for m in self.members])
        h = _P()
        code = self.L.mic_ensemble_create(ctypes.byref(h), arr, len(self.members))
        if code:
            raise MicError(code, "mic_ensemble_create")
        self.h = h

    def autotune(self, dt_disp=None, dt_thermal=None, subgrid_stress=1, steps=2):
        """mic_ensemble_autotune: members' launch shapes and the issue order of their steps;
        member states left unchanged.  Returns the order."""
        n = len(self.members)
        dd = np.ascontiguousarray(dt_disp if dt_disp is not None else [m.wl.dt for m in self.members], dtype=np.float64)
        dth = np.ascontiguousarray(dt_thermal if dt_thermal is not None else [m.wl.dt_thermal for m in self.members],
                                   dtype=np.float64)
        out = (ctypes.c_int * n)()
        code = self.L.mic_ensemble_autotune(self.h, _dp(dd), _dp(dth), subgrid_stress, steps, out)
        if code:
            raise MicError(code, "mic_ensemble_autotune")
        return list(out)

    def set_schedule(self, groups=4, tile_mult=4, persistent=True, chunked=2):
        """mic_ensemble_set_schedule: groups 0 = per-member kernels on member streams; 1..8 = batch
        groups, one kernel per marker pass per group; tile size in blocks' worth of markers and the
        persistent grid's walk (chunked 0 round-robin, 1 contiguous runs, 2 shared counter)."""
        code = self.L.mic_ensemble_set_schedule(self.h, int(groups), int(tile_mult), 1 if persistent else 0,
                                                int(chunked))
        if code:
            raise MicError(code, "mic_ensemble_set_schedule")

    def schedule(self):
        v = [ctypes.c_int(0) for _ in range(4)]
        code = self.L.mic_ensemble_get_schedule(self.h, *[ctypes.byref(x) for x in v])
        if code:
            raise MicError(code, "mic_ensemble_get_schedule")
        return {"groups": v[0].value, "tile_mult": v[1].value, "persistent": bool(v[2].value),
                "walk": ("round_robin", "runs", "counter")[v[3].value]}

    def step(self, dt_disp=None, dt_thermal=None, subgrid_stress=1, graph=True):
        n = len(self.members)
        dd = np.ascontiguousarray(dt_disp if dt_disp is not None else [m.wl.dt for m in self.members], dtype=np.float64)
        dth = np.ascontiguousarray(dt_thermal if dt_thermal is not None else [m.wl.dt_thermal for m in self.members],
                                   dtype=np.float64)
        assert len(dd) == n and len(dth) == n
        code = self.L.mic_ensemble_step(self.h, _dp(dd), _dp(dth), subgrid_stress, 1 if graph else 0)
        if code:
            raise MicError(code, "mic_ensemble_step")

    def synchronize(self):
        code = self.L.mic_ensemble_synchronize(self.h)
        if code:
            raise MicError(code, "mic_ensemble_synchronize")

    def launch_count(self):
        a, b = ctypes.c_int64(0), ctypes.c_int64(0)
        self.L.mic_ensemble_launch_count(self.h, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def stream(self):
        s = _P()
        self.L.mic_ensemble_get_stream(self.h, ctypes.byref(s))
        return s.value

    def close(self):
        if getattr(self, "h", None):
            self.L.mic_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def subduction_timestep_many(problems, topts, elapsed=None, max_threads=0):
    """One mic_subduction_timestep on every problem at once (independent Monte-Carlo members, each
    on its own stream, stepped from host threads side by side).  Returns the reports as dicts."""
    from .mic_types import TimestepOptions, TimestepReport

    n = len(problems)
    L = problems[0].L
    hs = (ctypes.c_void_p * n)(*[P.h for P in problems])
    opts = (TimestepOptions * n)(*topts)
    reps = (TimestepReport * n)()
    codes = (ctypes.c_int * n)()
    el = np.ascontiguousarray(np.zeros(n) if elapsed is None else elapsed, dtype=np.float64)
    e = L.mic_subduction_timestep_many(hs, n, opts, _dp(el), reps, codes, max_threads)
    for P in problems:
        P.n = P._count()
    if e:
        raise MicError(e, "mic_subduction_timestep_many (member codes %s)" % list(codes))
    return [r.as_dict() for r in reps]
