"""Build recipe for libpbf103.so (CUDA kernels + C ABI) for sm_103a.

Compiles each translation unit with nvcc in parallel and links one shared
library in-tree (``fluid-simulator_gb300/_build/libpbf103.so``).  No cmake, one
-gencode, a few seconds per unit.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libpbf103.so"
LIB_PATH = os.path.join(BUILD_DIR, LIB_NAME)

SOURCES = ["pbf_kernels.cu", "pbf_sort.cu", "pbf_solver.cu", "pbf_stages.cu", "pbf_noalloc.cu",
           "pbf_adjoint.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xcompiler", "-Wall", "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE,
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libpbf103")


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, INCLUDE):
        for root, _, files in os.walk(d):
            for f in files:
                m = max(m, os.path.getmtime(os.path.join(root, f)))
    return max(m, os.path.getmtime(__file__))


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile and link libpbf103.so; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _deps_mtime():
        return LIB_PATH
    cc = nvcc()
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [cc] + NVCC_FLAGS + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "--cudart=static", "-o", tmp] + objs + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


SHIM_BENCH_SRC = os.path.join(PKG_DIR, "cpp", "reference_scene_bench.cpp")
SHIM_BENCH = os.path.join(BUILD_DIR, "reference_scene_bench")


def build_shim_bench(force: bool = False) -> str:
    """Compile the reference-scene driver (cpp/reference_scene_bench.cpp)
    against the C++ shim with g++, linked to libpbf103.so; returns its path.
    Floating-point contraction is off so the scene's coordinates are the
    single-precision products and sums the reference's driver computes."""
    lib = build()
    if (not force and os.path.exists(SHIM_BENCH) and
            os.path.getmtime(SHIM_BENCH) >= max(os.path.getmtime(lib),
                                                os.path.getmtime(SHIM_BENCH_SRC))):
        return SHIM_BENCH
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    tmp = SHIM_BENCH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", INCLUDE, "-I", cuda_inc,
           SHIM_BENCH_SRC, "-o", tmp, lib, "-Wl,-rpath," + BUILD_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for %s:\n%s%s" % (SHIM_BENCH_SRC, r.stdout, r.stderr))
    os.replace(tmp, SHIM_BENCH)
    return SHIM_BENCH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_shim_bench(force=True))
