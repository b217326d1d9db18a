"""The C-ABI boundary without a GPU: both builds of the library load with every symbol
resolved and export every entry point that include/mic_gb300.h declares; struct layouts of
the public records match the reference's (checked in test_oracle_pin)."""
import ctypes
import os
import re

import pytest

from fvmic2d_gb300 import build, gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    src = open(os.path.join(ROOT, "include", "mic_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|void|int64_t|double|char)\s*\**\s*(mic_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def libs():
    build.build(variants=list(build.VARIANTS))
    # RTLD_NOW (ctypes' default mode adds it): an unresolved symbol fails here, not at first call
    return {name: ctypes.CDLL(build.lib_path(name), mode=os.RTLD_NOW | os.RTLD_LOCAL) for name in build.VARIANTS}


def test_header_declares_the_reference_entry_points():
    names = declared_entry_points()
    for fn in ["mic_find_marker_cells", "mic_project_markers_nodes_all2", "mic_project_marker_field_to_nodes",
               "mic_project_nodal_field_to_markers", "mic_check_plastic_yielding", "mic_update_viscosity",
               "mic_limit_viscosity", "mic_update_marker_strain_pressure", "mic_update_global_strain_rate_residual",
               "mic_check_convergence", "mic_subgrid_stress_changes", "mic_update_marker_stress",
               "mic_subgrid_temperature_changes", "mic_advect_markers_rk", "mic_bin_sort_noalloc"]:
        assert fn in names, fn


def test_libraries_export_every_declared_entry_point(libs):
    names = declared_entry_points()
    assert len(names) > 50
    for lib_name, L in libs.items():
        missing = [n for n in names if not hasattr(L, n)]
        assert not missing, (lib_name, missing)


def test_python_binding_covers_the_header():
    assert set(gpu.SIGNATURES) == set(declared_entry_points())


def test_create_without_device_fails_loudly(libs):
    """No GPU here: the product path reports MIC_ERR_NO_DEVICE instead of falling back."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = gpu.load()
    h = ctypes.c_void_p()
    x = (ctypes.c_double * 7)(-2.0, -1.0, 0.0, 1.0, 2.0, 3.0, 4.0)  # two ghost entries on each side
    xp = ctypes.cast(ctypes.byref(x, 2 * 8), ctypes.POINTER(ctypes.c_double))
    rc = L.mic_create(ctypes.byref(h), 0, None, 3, 3, 2.0, 2.0, xp, xp, 16)
    assert rc == 9  # MIC_ERR_NO_DEVICE
