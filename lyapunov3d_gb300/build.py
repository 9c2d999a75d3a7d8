"""Build the in-tree shared library lyapunov3d_gb300/_lib/liblyap_gb300.so.

nvcc compiles the CUDA translation units for sm_103a only (one -gencode),
g++ the host scene code; the translation units compile in parallel and the
library links the CUDA runtime statically, so it loads with nothing but the
driver.  Floating-point contraction is off everywhere (-fmad=false,
-ffp-contract=off): the per-ray arithmetic must round exactly like the
reference's host build; the lambda loop's fused multiply-adds are explicit.

    python -m lyapunov3d_gb300.build [--force] [--verbose]
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "liblyap_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["lyap_render.cu", "lyap_volume.cu", "lyap_capi.cu", "lyap_probe.cu", "lyap_noalloc.cu"]
CXX_SOURCES = ["lyap_scene.cpp"]
HEADERS = ["lyap_device.cuh", "lyap_internal.h"]


def nvcc_path():
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found (set NVCC or put /usr/local/cuda/bin on PATH)")


def nvcc_flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
                   "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}",
                   *extra]


def _deps():
    return ([os.path.join(CSRC, f) for f in CUDA_SOURCES + CXX_SOURCES + HEADERS] +
            [os.path.join(INCLUDE, "lyap_gb300.h"), os.path.join(INCLUDE, "lyap_kernel.hpp"), __file__])


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps() if os.path.exists(p))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = nvcc_path()
    jobs = []
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    for f in CUDA_SOURCES:
        obj = os.path.join(OBJDIR, f + ".o")
        jobs.append([nvcc, *nvcc_flags(extra), "-c", os.path.join(CSRC, f), "-o", obj])
    for f in CXX_SOURCES:
        obj = os.path.join(OBJDIR, f + ".o")
        jobs.append([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                     "-fno-fast-math", f"-I{INCLUDE}", f"-I{CSRC}", "-I/usr/local/cuda/include", "-c",
                     os.path.join(CSRC, f), "-o", obj])
    logs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            logs.append(out)
    objs = [os.path.join(OBJDIR, f + ".o") for f in CUDA_SOURCES + CXX_SOURCES]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs], verbose)
    os.replace(tmp, LIB)
    if ptxas_verbose:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
          ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
