"""The header-only C++ shim (include/pbf103/pbf_solver.hpp) compiles like code
written for the reference's PBFSolver and throws the reference's exception types.
"""

import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def build_shim_check(tmp_path, pbf):
    lib = pbf.load()
    exe = os.path.join(str(tmp_path), "shim_check")
    inc_cuda = "/usr/local/cuda/include"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", inc_cuda,
           os.path.join(ROOT, "tests", "cpp", "shim_check.cpp"), "-o", exe,
           pbf.library_path(), "-Wl,-rpath," + os.path.dirname(pbf.library_path())]
    subprocess.check_call(cmd)
    del lib
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_shim_cpu_validation(tmp_path, pbf):
    exe = build_shim_check(tmp_path, pbf)
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout


@pytest.mark.gpu
def test_shim_gpu_scenarios(tmp_path, pbf):
    exe = build_shim_check(tmp_path, pbf)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout


def _shim_bench(pbf):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "_pbf103_build_t", os.path.join(ROOT, "fluid-simulator_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build_shim_bench()


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_reference_scene_driver_builds_the_same_scene(tmp_path, pbf, scenes):
    """The C++ driver of the reference benchmark scene (written against the
    shim) starts from the same particles as the Python scene builder, bit for
    bit (benchmark/pbf_benchmark.cu:85-114)."""
    import numpy as np
    exe = _shim_bench(pbf)
    out = os.path.join(str(tmp_path), "scene.bin")
    subprocess.check_call([exe, "--dump", out], timeout=60)
    got = np.fromfile(out, np.float32).reshape(-1, 4)
    want = scenes.reference_benchmark()[0]
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_reference_scene_driver_runs(pbf):
    """The shim driver runs the reference benchmark protocol end to end."""
    import json
    exe = _shim_bench(pbf)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["particles"] == 262144 and d["substeps"] == 2 and len(d["runs_ms"]) == 5
    assert d["ms_per_frame"] > 0.0


def test_reference_benchmark_builds_unchanged_on_the_shim(tmp_path, pbf):
    """The reference's own benchmark driver compiles, unmodified, against the
    shim through the forwarding header include/compat/pbf/pbf_solver.hpp and
    links libpbf103.so (needs the reference tree; a build check only)."""
    import sys
    sys.path.insert(0, ROOT)
    from oracle import build_ref
    out = os.path.join(str(tmp_path), "pbf_benchmark_on_shim")
    if not build_ref.compile_benchmark_on_shim(pbf.library_path(), os.path.join(ROOT, "include"),
                                               out):
        pytest.skip("reference tree not present")
    assert os.path.exists(out)
