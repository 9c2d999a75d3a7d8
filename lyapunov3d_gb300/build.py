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
CUDA_SOURCES = ["lyap_render.cu", "lyap_volume.cu", "lyap_capi.cu", "lyap_probe.cu", "lyap_noalloc.cu", "lyap_precise.cu", "lyap_batch.cu", "lyap_net.cu",
                "lyap_f64.cu"]
CXX_SOURCES = ["lyap_scene.cpp", "lyap_jit.cpp", "lyap_preset.cpp", "lyap_io.cpp"]
# the reference front-ends' command-line equivalents (linked against the library)
CLI_SOURCES = ["lyap_calculate.cpp", "lyap_frame.cpp"]
CLIDIR = os.path.join(PKG, "cli")
HEADERS = ["lyap_device.cuh", "lyap_internal.h", "lyap_jobs.h", "lyap_kernels.cuh", "lyap_jit.h", "lyap_net.cuh",
           "lyap_tc.cuh"]
# headers NVRTC compiles at run time (embedded into the library), and minimal
# stand-ins for the two C headers they include
JIT_HEADERS = [("lyap_gb300.h", "INCLUDE"), ("lyap_jobs.h", "CSRC"), ("lyap_device.cuh", "CSRC"),
               ("lyap_kernels.cuh", "CSRC")]
JIT_STUBS = {
    "stdint.h": ("#pragma once\n"
                 "typedef signed char int8_t; typedef short int16_t; typedef int int32_t;\n"
                 "typedef long long int64_t; typedef unsigned char uint8_t; typedef unsigned short uint16_t;\n"
                 "typedef unsigned int uint32_t; typedef unsigned long long uint64_t;\n"),
    "stddef.h": ("#pragma once\n"
                 "typedef unsigned long size_t; typedef long ptrdiff_t;\n"
                 "#define offsetof(t, m) __builtin_offsetof(t, m)\n"
                 "#ifndef NULL\n#define NULL 0\n#endif\n"),
}


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


def cli_binary(src):
    return os.path.join(LIBDIR, os.path.splitext(src)[0])


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    if not all(os.path.getmtime(p) <= t for p in _deps() if os.path.exists(p)):
        return False
    for c in CLI_SOURCES:
        b = cli_binary(c)
        if not os.path.exists(b) or os.path.getmtime(b) < max(t, os.path.getmtime(os.path.join(CLIDIR, c))):
            return False
    return True


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def write_jit_sources(path):
    """A C++ file holding the JIT headers as raw string literals (lyap_jit.cpp reads them)."""
    names, texts = [], []
    for name, where in JIT_HEADERS:
        with open(os.path.join(INCLUDE if where == "INCLUDE" else CSRC, name)) as f:
            names.append(name)
            texts.append(f.read())
    for name, text in JIT_STUBS.items():
        names.append(name)
        texts.append(text)
    out = ["// generated by lyapunov3d_gb300/build.py: device headers for run-time compilation", "namespace lyapgb {",
           f"extern const int kJitHeaderCount = {len(names)};", "extern const char *const kJitHeaderNames[] = {"]
    out += [f'    "{n}",' for n in names] + ["};", "extern const char *const kJitHeaderSources[] = {"]
    for t in texts:
        assert ")LYAPSRC\"" not in t
        out.append('    R"LYAPSRC(' + t + ')LYAPSRC",')
    out += ["};", "}  // namespace lyapgb", ""]
    data = "\n".join(out)
    if not os.path.exists(path) or open(path).read() != data:
        with open(path, "w") as f:
            f.write(data)
    return path


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
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    jit_src = write_jit_sources(os.path.join(OBJDIR, "lyap_jit_sources.cpp"))
    for f in CXX_SOURCES + ["lyap_jit_sources.cpp"]:
        obj = os.path.join(OBJDIR, f + ".o")
        src = jit_src if f == "lyap_jit_sources.cpp" else os.path.join(CSRC, f)
        jobs.append([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                     "-fno-fast-math", f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda_inc}", "-c", src, "-o", obj])
    logs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            logs.append(out)
    objs = [os.path.join(OBJDIR, f + ".o") for f in CUDA_SOURCES + CXX_SOURCES + ["lyap_jit_sources.cpp"]]
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-ldl"], verbose)
    os.replace(tmp, LIB)
    cli_jobs = [[os.environ.get("CXX", "g++"), "-O2", "-std=c++17", f"-I{INCLUDE}", os.path.join(CLIDIR, c), "-o",
                 cli_binary(c), f"-L{LIBDIR}", "-llyap_gb300", "-Wl,-rpath,$ORIGIN"] for c in CLI_SOURCES]
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(cli_jobs)) as ex:
        list(ex.map(lambda c: _run(c, verbose), cli_jobs))
    if ptxas_verbose:
        print("\n".join(l for l in logs if l.strip()))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
          ptxas_verbose="--ptxas" in sys.argv)
    print(LIB)
