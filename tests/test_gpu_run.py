"""The whole subduction program (main_subduction.c:176-460) on the device through
fvmic2d_gb300.run_subduction: set-up and two time steps against the reference's own routines
called in main's order with host sparse LU solves (golden vectors), and the command-line driver
with its marker files."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from fvmic2d_gb300 import gpu
from fvmic2d_gb300 import run_subduction as RS
from fvmic2d_gb300.mic_types import MARKER_DTYPE
from tests.test_gpu_timestep import FIELD_RTOL, _fields
from tests.timestep_case import run_case

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _close(got, ref, scale_mult=1.0):
    gf, rf = _fields(got), _fields(ref)
    worst = {}
    for k, tol in FIELD_RTOL.items():
        scale = np.max(np.abs(rf[k]))
        worst[k] = np.max(np.abs(gf[k] - rf[k])) / scale
    for k, tol in FIELD_RTOL.items():
        assert worst[k] <= tol * scale_mult, (k, worst)


def test_setup_and_two_steps_match_reference():
    """set-up: the uniform marker lattice bit for bit, the van Keken initial conditions and the
    temperature projected back from the nodes within 1e-12 of the field's largest magnitude;
    each step: the time-step report and the marker fields within the single-step tolerances"""
    z = np.load(os.path.join(GOLDEN, "subduction_run.npz"))
    wl, topt, nmx, nmy, steps = run_case()
    cap = int(1.5 * nmx * nmy * (wl.grid.NX - 1) * (wl.grid.NY - 1)) + 64
    P = gpu.MicProblem(wl, capacity=cap)
    n = RS.setup(P, topt.sub, nmx, nmy)
    ref = z["setup"].view(MARKER_DTYPE)
    assert n == len(ref)
    got = P.markers
    for f in ("X", "Y", "Mat", "cellX", "cellY"):
        assert np.array_equal(got[f], ref[f]), f
    for f in ("T", "rho", "eta", "mu"):
        assert np.max(np.abs(got[f] - ref[f])) <= 1e-12 * np.max(np.abs(ref[f])), f

    seen = []
    _, reps = RS.run(P, topt, steps, on_step=lambda it, rep, t: seen.append(P.markers))
    assert len(reps) == steps
    for i, rep in enumerate(reps):
        assert rep["stopped"] == 0
        for k in ("plastic_iterations", "is_yielding", "converged", "thermal_resolves", "markers_added"):
            assert rep[k] == int(z["rep%d_%s" % (i, k)]), (i, k)
        for k in ("dt", "displacement_dt", "Kbond", "Kcont", "max_T", "max_temp_change", "max_abs_sxx", "nusselt",
                  "vrms"):
            ref_v = float(z["rep%d_%s" % (i, k)])
            assert abs(rep[k] - ref_v) <= 1e-9 * abs(ref_v), (i, k, rep[k], ref_v)
        _close(seen[i], z["step%d" % i].view(MARKER_DTYPE))
    P.close()


def test_command_line_driver_writes_marker_files(tmp_path):
    """python -m fvmic2d_gb300.run_subduction: one JSON line per step and a closing line; the
    marker files it saves restart a fresh context at the saved time with the saved markers"""
    out = tmp_path / "out"
    cmd = [sys.executable, "-m", "fvmic2d_gb300.run_subduction", "--nx-cells", "32", "--ny-cells", "8",
           "--steps", "3", "--save-every", "2", "--out", str(out)]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert [l["step"] for l in lines[:-1]] == [0, 1, 2]
    last = lines[-1]
    assert last["steps"] == 3 and last["markers_at_setup"] == 16 * 32 * 8
    assert abs(last["elapsed_time"] - sum(l["dt"] for l in lines[:-1])) <= 1e-12 * last["elapsed_time"]
    assert all(np.isfinite([l["nusselt"], l["vrms"], l["residual"]]).all() for l in lines[:-1])
    assert sorted(os.listdir(out)) == ["Markers.0.0", "Markers.0.2"]

    wl, topt, nmx, nmy, _ = run_case()
    Q = gpu.MicProblem(wl, capacity=4 * 16 * 32 * 8)
    t = Q.restartFromMarkers(str(out / "Markers.0.2"))
    assert abs(t - last["elapsed_time"]) <= 1e-12 * t
    m = Q.markers
    assert len(m) >= 16 * 32 * 8 - 64
    assert np.all(np.isfinite(m["T"])) and m["T"].min() > 200.0 and m["T"].max() < 1700.0
    Q.close()
