"""Build recipe for libmic_gb300.so (CUDA, sm_103a only).

Two variants are compiled from the same sources:
  libmic_gb300.so        -- the product build (FMA contraction on)
  libmic_gb300_exact.so  -- -fmad=false: every FP64 expression rounds like the reference's
                            host C (compiled with -ffp-contract=off), used by the parity tests
Translation units compile in parallel; nothing here needs cmake or torch.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["mic_context.cu", "mic_bin_sort.cu", "mic_project.cu", "mic_marker_passes.cu", "mic_creep.cu",
           "mic_creep_tc.cu", "mic_ensemble.cu", "mic_density.cu", "mic_grid.cu", "mic_io.cu", "mic_systems.cu",
           "mic_band_lu.cu", "mic_timestep.cu", "mic_autotune.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
VARIANTS = {"libmic_gb300.so": ["-fmad=true"], "libmic_gb300_exact.so": ["-fmad=false", "-DMIC_EXACT=1"]}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path(name="libmic_gb300.so"):
    return os.path.join(HERE, name)


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return hdrs


def _stale(target, inputs):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in inputs)


def _compile(args):
    src, obj, flags = args
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
           *flags, "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
    with open(obj + ".ptxas.txt", "w") as f:
        f.write(r.stderr)
    return obj


def build(force=False, variants=None, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    variants = variants or list(VARIANTS)
    deps = _deps()
    jobs_list, links = [], []
    for name in variants:
        flags = VARIANTS[name]
        tag = name.replace(".so", "")
        objs = []
        for s in SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(BUILD, tag + "_" + s.replace(".cu", ".o"))
            if force or _stale(obj, [src] + deps):
                jobs_list.append((src, obj, flags))
            objs.append(obj)
        links.append((name, objs))
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_list), os.cpu_count() or 4)) as ex:
            list(ex.map(_compile, jobs_list))
    out = []
    for name, objs in links:
        target = lib_path(name)
        if force or _stale(target, objs):
            cmd = [nvcc(), *ARCH, "-shared", "-o", target, *objs, "-lcudart"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed for %s:\n%s" % (name, r.stderr))
        out.append(target)
    return out


if __name__ == "__main__":
    for p in build(force=True):
        print(p)
