"""Shared fixtures: the package under test, the CPU oracle, reference parameter sets."""

from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "fluid_simulator_gb300"


def load_pkg():
    """Import the package directory ``fluid-simulator_gb300`` (its name has a hyphen)."""
    if PKG_NAME in sys.modules:
        return sys.modules[PKG_NAME]
    pkg_dir = os.path.join(ROOT, "fluid-simulator_gb300")
    spec = importlib.util.spec_from_file_location(
        PKG_NAME, os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[PKG_NAME] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpbf103.so")


@pytest.fixture(scope="session")
def pbf():
    return load_pkg()


@pytest.fixture(scope="session")
def scenes():
    load_pkg()
    return importlib.import_module(PKG_NAME + ".scenes")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.lib()
    return O


PI_F = np.float32(3.14159265358979323846)


def self_density(mass: float, h: float) -> float:
    """selfDensity of test/test_pbf_solver.cu:39-42 (float arithmetic)."""
    return float(np.float32(mass) * np.float32(315.0) /
                 (np.float32(64.0) * PI_F * np.float32(h) ** np.float32(3.0)))


def pair_density(mass: float, distance: float, h: float) -> float:
    """pairDensityContribution of test/test_pbf_solver.cu:44-51."""
    r2 = np.float32(h) * np.float32(h)
    d = r2 - np.float32(distance) * np.float32(distance)
    return float(np.float32(mass) * np.float32(315.0) /
                 (np.float32(64.0) * PI_F * np.float32(h) ** np.float32(9.0)) * d * d * d)


def valid_params() -> dict:
    """validParams of test/test_pbf_solver.cu:17-37."""
    return dict(dt=0.1, restDensity=float(np.float32(315.0) / (np.float32(64.0) * PI_F)),
                particleMass=1.0, particleRadius=1.0, collisionRestitution=0.0,
                collisionFriction=0.03, smoothingRadius=1.0, lambdaEpsilon=0.01,
                solverIterations=1, substeps=1, gravity=(0.0, -9.8, 0.0), scorrK=0.0, scorrN=0,
                scorrDeltaQ=0.0, xsphViscosity=0.0, vorticityStrength=0.0)


def collision_params() -> dict:
    """collisionParams of test/test_pbf_solver.cu:85-97."""
    p = valid_params()
    p.update(dt=0.1, particleRadius=0.25, smoothingRadius=0.5,
             restDensity=self_density(1.0, 0.5), solverIterations=4, substeps=1,
             gravity=(0.0, 0.0, 0.0), collisionRestitution=0.0, collisionFriction=0.0)
    return p


SOLVER_MIN = (-2.0, -2.0, -2.0)  # initializeSolver bounds, test/test_pbf_solver.cu:53-61
SOLVER_MAX = (12.0, 12.0, 12.0)


def f4(*rows):
    return np.array(rows, dtype=np.float32).reshape(-1, 4)
