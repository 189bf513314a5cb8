"""Recipe: the reference's CUDA kernels, compiled from its own sources.

TEST INFRASTRUCTURE ONLY.  Compiles the five kernel translation units of the
reference (DusanCojic/Fluid-Simulator, src/pbf/*.cu) exactly as its benchmark
workflow does (Release: -O3 -DNDEBUG, benchmark/profile.py:609-613), for
sm_103a, one fatbin per unit, into oracle/_ref/.  Only device code is kept
(a fatbin, no host code), so the output travels to the Arm GPU machine; the
driver in oracle/ref_driver.cu loads it there.  Nothing is copied: the
sources are read where they lie.

build_if_possible() is a no-op when the reference tree is absent (the GPU machine
uses the fatbins built here).  The reference tree is taken from the
PBF_REFERENCE_DIR environment variable, or from `--reference DIR` when this
recipe runs as a script; without either, the recipe looks in the one place
the reference is checked out for this project's checker builds.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE = os.environ.get("PBF_REFERENCE_DIR") or "/root/reference"
UNITS = ["integration", "neighbors", "pbf_solver_kernels", "collision_kernels", "spatial_grid"]
FLAGS = ["-fatbin", "-std=c++20", "-O3", "-DNDEBUG", "-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def fatbin_path(unit: str) -> str:
    return os.path.join(OUT, unit + ".fatbin")


def available() -> bool:
    return all(os.path.exists(fatbin_path(u)) for u in UNITS)


def build(force: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    inc = os.path.join(REFERENCE, "include")

    def one(unit):
        src = os.path.join(REFERENCE, "src", "pbf", unit + ".cu")
        out = fatbin_path(unit)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            return out
        tmp = out + ".tmp"
        subprocess.check_call([nvcc()] + FLAGS + ["-I", inc, src, "-o", tmp])
        os.replace(tmp, out)
        return out

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(one, UNITS))


def build_if_possible() -> bool:
    if os.path.isdir(os.path.join(REFERENCE, "src", "pbf")):
        build()
        return True
    return available()


def compile_benchmark_on_shim(lib_path: str, include_dir: str, out_path: str) -> bool:
    """Compiles the reference's benchmark driver (benchmark/pbf_benchmark.cu),
    unmodified, against this repository's C++ shim (include_dir/compat puts
    the shim at "pbf/pbf_solver.hpp") and links lib_path.  Returns False when
    the reference tree is absent.  A build check: the binary is not run."""
    src = os.path.join(REFERENCE, "benchmark", "pbf_benchmark.cu")
    if not os.path.exists(src):
        return False
    subprocess.check_call([nvcc(), "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I", os.path.join(include_dir, "compat"), "-I", include_dir, src,
                           "-o", out_path, lib_path, "-Xlinker",
                           "-rpath=" + os.path.dirname(lib_path)])
    return True


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="reference source tree")
    a = ap.parse_args()
    if a.reference:
        REFERENCE = a.reference
    build(force=True)
    print("\n".join(fatbin_path(u) for u in UNITS))
