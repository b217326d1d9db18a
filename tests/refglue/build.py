"""Build recipe for the reference-side binding's test library (TEST INFRASTRUCTURE ONLY).

build_driver(): fvmic2d_gb300/refglue/fvmic2d_glue.c + tests/refglue/glue_driver.c + the
    petsc_lite stand-in, compiled against the stand-in fdcode.h and prototype headers
    (tests/refglue/standin/) and linked to libmic_gb300.so (product or FMA-free build):
    tests/refglue/_build/libgluedrv[_exact].so.  Needs only gcc and the built library.
compile_against_reference(ref_dir, obj): the binding compiled (not linked) against the reference's
    own fdcode.h and prototype headers, which checks each definition against the reference's
    declaration.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
GLUE = os.path.join(ROOT, "fvmic2d_gb300", "refglue", "fvmic2d_glue.c")
DRIVER = os.path.join(HERE, "glue_driver.c")
PLITE = os.path.join(ROOT, "oracle", "petsc_lite")
CFLAGS = ["-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-Wall", "-Werror=implicit-function-declaration",
          "-Werror=incompatible-pointer-types", "-Werror=int-conversion"]


def _cc():
    return os.environ.get("CC", "gcc")


def build_driver(exact=False):
    from fvmic2d_gb300 import build as fbuild

    lib_name = "libmic_gb300_exact.so" if exact else "libmic_gb300.so"
    lib = fbuild.lib_path(lib_name)
    if not os.path.exists(lib):
        raise RuntimeError(lib_name + " is not built")
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libgluedrv_exact.so" if exact else "libgluedrv.so")
    inc = ["-I" + os.path.join(HERE, "standin"), "-I" + os.path.join(PLITE, "include"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "fvmic2d_gb300", "refglue")]
    srcs = [GLUE, DRIVER, os.path.join(PLITE, "petsc_lite.c")]
    deps = srcs + [os.path.join(HERE, "standin", f) for f in os.listdir(os.path.join(HERE, "standin"))]
    deps += [os.path.join(ROOT, "fvmic2d_gb300", "refglue", "fvmic2d_glue.h"), lib]
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(p) for p in deps):
        return out
    cmd = [_cc(), *CFLAGS, "-shared", *inc, *srcs, "-o", out, lib, "-Wl,-rpath," + os.path.dirname(lib), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("glue driver build failed:\n" + r.stderr)
    return out


def compile_against_reference(ref_dir, obj):
    """The binding includes fdcode.h and the routines' prototype headers itself: with the reference
    tree first on the include path, the compiler checks each definition against the reference's
    own declaration (a mismatch is an error).  Returns the completed process."""
    inc = ["-I" + ref_dir, "-I" + os.path.join(PLITE, "include"), "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "fvmic2d_gb300", "refglue")]
    cmd = [_cc(), *CFLAGS, "-c", *inc, GLUE, "-o", obj]
    return subprocess.run(cmd, capture_output=True, text=True)
