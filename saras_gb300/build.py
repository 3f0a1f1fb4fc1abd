"""Build the GB300 library (saras_gb300/_build/libsaras_gb300.so) with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then linked
into one shared library that the ctypes layer and the C++ driver load.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsaras_gb300.so")
DRIVER = os.path.join(OUT, "saras_gb300_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: the FP64 kernels must round every product and sum exactly as
# the reference expressions do (kernels that want fused multiply-adds call
# fma() explicitly); -ffp-contract=off does the same for the host code (grid
# metrics), which Arm compilers would otherwise contract.
COMMON = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]
UNITS = ["capi.cu", "fields.cu", "multigrid.cu", "unet.cu"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "saras_gb300.h"))
    return hs


def _compile(unit, extra, verbose):
    src = os.path.join(SRC, unit)
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    if not _stale(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, ptxas_info=False):
    os.makedirs(OUT, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u, extra, verbose or ptxas_info), UNITS))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    drv_src = os.path.join(SRC, "saras_main.cc")
    if os.path.exists(drv_src) and _stale(DRIVER, [drv_src, LIB]):
        cmd = ["g++", "-O2", "-std=c++17", "-o", DRIVER, drv_src, "-I" + os.path.join(os.path.dirname(HERE), "include"),
               "-L" + OUT, "-lsaras_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
