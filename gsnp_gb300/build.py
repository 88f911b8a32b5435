"""Build the native libraries (sm_103a kernels + host code).

Every translation unit is compiled in parallel into gsnp_gb300/_build/ and
linked with a static CUDA runtime into
  gsnp_gb300/_lib/libgsnp_gb300.so   the C ABI of include/gsnp_gb300.h;
  gsnp_gb300/_lib/libgsnp_backend.so the reference's C++ backend functions
                                     (include/gsnp_backend.h) for host code
                                     written against them;
  gsnp_gb300/_lib/gsnp               the command-line caller (cli.cpp) over
                                     the C ABI;
  gsnp_gb300/_lib/gsnp_decompress    the -C decompressor command
                                     (decompress_main.cpp) over the C ABI.
Floating point is pinned: device code with --fmad=false (no fused
multiply-add the source does not spell out), host code with
-ffp-contract=off.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libgsnp_gb300.so")
BACKEND_LIB = os.path.join(LIBDIR, "libgsnp_backend.so")
# translation units of each library
BACKEND_ONLY = {"compat.cu"}
BACKEND_UNITS = {"compat.cu", "dict.cu", "tables.cpp"}
CLI_UNIT = "cli.cpp"
CLI = os.path.join(LIBDIR, "gsnp")
DECOMPRESS_UNIT = "decompress_main.cpp"
DECOMPRESS = os.path.join(LIBDIR, "gsnp_decompress")
COMMANDS = {CLI_UNIT: CLI, DECOMPRESS_UNIT: DECOMPRESS}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-Wall",
             "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")


def _sources():
    srcs = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cpp"):
            srcs.append(os.path.join(CSRC, f))
    return srcs


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile all sources; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    incs = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if not force and not _newer(obj, [src] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [_nvcc()] + NVCC_FLAGS + incs + ["-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + incs + ["-I" + _cuda_include(), "-c", src, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append(cmd[-3])
    if failed:
        raise RuntimeError("compilation failed: " + ", ".join(failed))
    lib_objs = [o for o in objs if os.path.basename(o)[:-2] not in COMMANDS]
    for lib, units in ((LIB, [o for o in lib_objs if os.path.basename(o)[:-2] not in BACKEND_ONLY]),
                       (BACKEND_LIB, [o for o in lib_objs if os.path.basename(o)[:-2] in BACKEND_UNITS])):
        if force or jobs or not os.path.exists(lib):
            cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", lib] + units
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    for unit, exe in COMMANDS.items():
        obj = os.path.join(BUILD, unit + ".o")
        if force or _newer(exe, [obj, LIB]):
            cmd = ["g++", "-o", exe, obj, "-L" + LIBDIR, "-lgsnp_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
