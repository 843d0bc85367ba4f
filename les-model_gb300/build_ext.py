"""Builds les-model_gb300/libles_gb300.so (the CUDA kernels + C ABI) for
sm_103a with nvcc, translation units in parallel.

FP64 translation units are compiled with -fmad=false so that every a*b+c
rounds twice, like the reference's x86-64 -O2 build (which has no FMA); the
mixed-precision unit may contract.

    python les-model_gb300/build_ext.py [--force]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libles_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags
UNITS = {
    "les_ctx.cu": ["-fmad=false"],
    "les_physics.cu": ["-fmad=false"],
    "les_physics32.cu": [],
    "les_pressure.cu": ["-fmad=false"],
    "les_wavefront.cu": ["-fmad=false"],
    "les_mixed.cu": [],
    "les_fused.cu": [],
    "les_col.cu": [],
    "les_col_sj32.cu": [],
    "les_col_sj64.cu": [],
    "les_col_sj128.cu": [],
    "les_col_sj256.cu": [],
    "les_ensemble.cu": [],
    "les_tune.cu": [],
    "les_adjoint.cu": ["-fmad=false"],
    "les_io.cu": ["-fmad=false"],
    "les_step.cu": ["-fmad=false"],
    "les_noalloc.cu": ["-fmad=false"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "les_gb300.h"))
    files += [os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host"))]
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    base = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC, *extra]

    def one(unit):
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = base + UNITS[unit] + ["-c", os.path.join(CSRC, unit), "-o", obj]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or p.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
        if p.returncode:
            raise RuntimeError("nvcc failed on %s" % unit)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(one, sorted(UNITS)))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode:
        sys.stderr.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    build_shim()
    return LIB


SHIM = os.path.join(HERE, "libles_shim.so")


def build_shim():
    """The reference-API shim (host/les_shim.cpp) over libles_gb300.so."""
    tmp = SHIM + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(HERE, "host"), os.path.join(HERE, "host", "les_shim.cpp"), "-L", HERE,
           "-lles_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode:
        sys.stderr.write(" ".join(cmd) + "\n" + p.stdout + p.stderr)
        raise RuntimeError("shim build failed")
    os.replace(tmp, SHIM)
    return SHIM


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force="--force" in sys.argv or bool(extra), verbose=v or bool(extra), extra=extra))
