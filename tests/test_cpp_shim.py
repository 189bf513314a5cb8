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
