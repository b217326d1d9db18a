"""Build recipe for the CPU oracle (test infrastructure only).

build_oracle(): compiles oracle/mic_oracle.c into oracle/liboracle.so (any host, gcc).
build_ref():    compiles fvmic2d's own hot-path sources against petsc_lite into
                oracle/_ref/libfvmic2d_ref.so, only where the reference tree exists.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_SO = os.path.join(HERE, "liboracle.so")
# the fvmic2d source tree: FVMIC2D_REFERENCE_DIR, else a checkout named "reference" beside this
# repository
REFERENCE_DIR = os.environ.get("FVMIC2D_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def build_oracle(force=False):
    src = os.path.join(HERE, "mic_oracle.c")
    hdrs = [os.path.join(HERE, "mic_oracle.h"), os.path.join(ROOT, "include", "mic_types.h")]
    if not force and os.path.exists(ORACLE_SO):
        newest = max(os.path.getmtime(p) for p in [src] + hdrs)
        if os.path.getmtime(ORACLE_SO) >= newest:
            return ORACLE_SO
    cmd = [
        os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-std=gnu99",
        "-ffp-contract=off", "-fno-fast-math",
        "-I" + os.path.join(ROOT, "include"), src, "-o", ORACLE_SO, "-lm",
    ]
    subprocess.run(cmd, check=True)
    return ORACLE_SO


def build_ref(reference_dir=REFERENCE_DIR):
    """Returns the library path, or None where the reference tree is absent."""
    if not os.path.isfile(os.path.join(reference_dir, "markerProjection.c")):
        return None
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh"), reference_dir], check=True,
                   stdout=subprocess.DEVNULL)
    return os.path.join(HERE, "_ref", "libfvmic2d_ref.so")


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref())
