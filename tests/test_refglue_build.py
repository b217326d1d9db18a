"""The reference-side binding (fvmic2d_gb300/refglue/fvmic2d_glue.c) without a GPU: it compiles
against fvmic2d's own headers -- every routine's definition meets the reference's declaration --
and the stand-in headers its GPU test builds with where the reference tree is absent have the
reference's record layouts, member for member.  The binding also links into its test driver
against the built library."""
import os
import subprocess
import sys

import pytest

from oracle import build as obuild
from tests.refglue import build as gbuild

REF = obuild.REFERENCE_DIR
needs_ref = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "fdcode.h")),
                               reason="fvmic2d source tree not present")

ROUTINES = ["allocateMarkers", "destroyMarkers", "resetMarkers", "distributeMarkersUniformInDomain",
            "findMarkerCells", "checkPlasticYielding", "checkMarkerDensity", "advectMarkersRK",
            "projectMarkersNodesFromScalar", "projectNodalFieldToMarkersS", "updateViscosity", "limitViscosity",
            "projectMarkersNodesAll2", "projectMarkerFieldToNodes", "updateMarkerStrainPressure",
            "updateGlobalStrainRateResidual", "getGlobalStrainRateResidual", "setGlobalStrainRateResidual",
            "checkConvergence", "subgridStressChanges", "updateMarkerStress", "subgridTemperatureChanges"]


def _defined_symbols(path):
    out = subprocess.run(["nm", "-g", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@needs_ref
def test_binding_compiles_against_the_reference_headers(tmp_path):
    obj = str(tmp_path / "glue.o")
    r = gbuild.compile_against_reference(REF, obj)
    assert r.returncode == 0, r.stderr[-4000:]
    missing = [f for f in ROUTINES if f not in _defined_symbols(obj)]
    assert not missing, missing


def _layout(tmp_path, include_dir, tag):
    exe = str(tmp_path / ("layout_" + tag))
    cmd = [os.environ.get("CC", "gcc"), "-std=gnu99", "-I" + include_dir,
           "-I" + os.path.join(gbuild.PLITE, "include"), "-I" + os.path.join(gbuild.ROOT, "include"),
           os.path.join(gbuild.HERE, "layout.c"), "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines()


@needs_ref
def test_standin_records_match_the_reference_layout(tmp_path):
    ref = _layout(tmp_path, REF, "ref")
    standin = _layout(tmp_path, os.path.join(gbuild.HERE, "standin"), "standin")
    assert len(ref) > 100
    diff = [(a, b) for a, b in zip(ref, standin) if a != b]
    assert ref == standin, diff[:10]


def test_binding_links_into_its_driver():
    path = gbuild.build_driver(exact=False)
    syms = _defined_symbols(path)
    missing = [f for f in ROUTINES + ["micMarkersToHost", "gd_create"] if f not in syms]
    assert not missing, missing
