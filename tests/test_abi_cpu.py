"""C-ABI checks that need no GPU.

* libpbf103.so loads and exports every function include/pbf103.h declares.
* Argument validation of PBFSolver::initialize / setParticles / collider
  setters / copy*ToHost (test/test_pbf_solver.cu:135-427,
  test/test_collision_system.cu:136-312) runs before any CUDA call, so the
  exception mapping is exercised through the real C ABI on the CPU.
"""

import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT, valid_params

HEADERS = [os.path.join(ROOT, "include", "pbf103.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(pbf_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_boundary():
    fns = declared_functions()
    for required in ("pbf_solver_create", "pbf_initialize", "pbf_set_particles", "pbf_step",
                     "pbf_run", "pbf_copy_positions", "pbf_copy_velocities", "pbf_set_spheres",
                     "pbf_set_boxes", "pbf_set_planes", "pbf_grid_build", "pbf_find_neighbors"):
        assert required in fns


def test_library_exports_every_declared_symbol(pbf):
    L = pbf.load()
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_version(pbf):
    assert "sm_103a" in pbf.version()


def expect(pbf, exc, fn, *args):
    with pytest.raises(exc):
        fn(*args)


def test_use_before_initialize(pbf):
    s = pbf.PBFSolver()
    one = np.zeros((1, 4), np.float32)
    with pytest.raises(pbf.LogicError):
        s.set_particles(one, one)
    with pytest.raises(pbf.LogicError):
        s.step()
    with pytest.raises(pbf.LogicError):
        s.run()
    with pytest.raises(pbf.OutOfRange):
        s.copy_positions_raw(None, 1)
    with pytest.raises(pbf.OutOfRange):
        s.copy_velocities_raw(None, 1)
    # Zero-count copies of an empty solver are fine, like the reference.
    s.copy_positions_raw(None, 0)


def test_walk_lanes_setting(pbf):
    """Lanes per particle of the walks: 0 (default), 1, 2, 4 or 8; anything
    else is rejected and leaves the setting unchanged."""
    s = pbf.PBFSolver()
    s.set_walk_lanes(2)
    assert s.walk_lanes() == 2
    for bad in (-1, 3, 16):
        with pytest.raises(pbf.InvalidArgument):
            s.set_walk_lanes(bad)
    assert s.walk_lanes() == 2
    s.set_walk_lanes(0)


def P(**kw):
    p = valid_params()
    p.update(kw)
    return p


def test_invalid_capacity_and_bounds(pbf):
    SP = pbf.SimulationParams
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize(0, (0, 0, 0), (1, 1, 1), SP(**P()))
    with pytest.raises(pbf.LengthError):
        s.initialize(2 ** 31, (0, 0, 0), (1, 1, 1), SP(**P()))
    with pytest.raises(pbf.InvalidArgument):
        s.initialize(8, (1, 0, 0), (1, 2, 2), SP(**P()))
    with pytest.raises(pbf.InvalidArgument):  # container narrower than a diameter
        s.initialize(8, (0, 0, 0), (1, 2, 1), SP(**P()))
    with pytest.raises(pbf.LengthError):      # grid axis beyond int range
        s.initialize(8, (0, 0, 0), (1e20, 2, 2), SP(**P(particleRadius=0.1)))


def test_invalid_compact_list_capacity(pbf):
    SP = pbf.SimulationParams
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize(8, (0, 0, 0), (1, 1, 1), SP(**P()), list_capacity=0)
    with pytest.raises(pbf.LengthError):
        s.initialize(8, (0, 0, 0), (1, 1, 1), SP(**P()), list_capacity=2 ** 32)
    with pytest.raises(pbf.InvalidArgument):
        s.initialize(8, (0, 0, 0), (1, 1, 1), SP(**P()), max_neighbors=0, list_capacity=64)
    with pytest.raises(pbf.InvalidArgument):  # validation still runs first
        s.initialize(8, (0, 0, 0), (1, 1, 1), SP(**P(dt=0.0)), list_capacity=64)


def test_adjoint_collider_validation(pbf):
    a = pbf.PBFAdjoint()
    with pytest.raises(pbf.InvalidArgument):
        a.set_spheres([((0.0, 0.0, 0.0), 0.0)])
    with pytest.raises(pbf.InvalidArgument):
        a.set_boxes([((0.0, 0.0, 0.0), (1.0, -1.0, 1.0))])
    with pytest.raises(pbf.InvalidArgument):
        a.set_planes([((0.0, 0.0, 0.0), (0.0, 0.0, 0.0))])
    a.close()


INVALID = [
    dict(dt=0.0), dict(dt=math.nan), dict(dt=1.4e-45, substeps=2),
    dict(restDensity=-1.0), dict(restDensity=math.inf),
    dict(particleMass=0.0), dict(particleMass=math.nan),
    dict(particleRadius=0.0), dict(particleRadius=math.inf),
    dict(collisionRestitution=-0.01), dict(collisionRestitution=1.01),
    dict(collisionRestitution=math.nan), dict(collisionRestitution=math.inf),
    dict(collisionFriction=-0.01), dict(collisionFriction=1.01),
    dict(collisionFriction=math.nan), dict(collisionFriction=math.inf),
    dict(smoothingRadius=-1.0), dict(smoothingRadius=math.inf),
    dict(lambdaEpsilon=0.0), dict(lambdaEpsilon=-0.01), dict(lambdaEpsilon=math.nan),
    dict(gravity=(math.inf, -9.8, 0)), dict(gravity=(0, math.nan, 0)),
    dict(gravity=(0, -9.8, -math.inf)),
    dict(solverIterations=0), dict(solverIterations=-1), dict(substeps=0), dict(substeps=-1),
    dict(vorticityStrength=-0.01), dict(vorticityStrength=math.inf),
    dict(xsphViscosity=-1.0), dict(scorrK=0.1, scorrN=0), dict(scorrK=0.1, scorrN=4,
                                                              scorrDeltaQ=1.0),
]


@pytest.mark.parametrize("bad", INVALID, ids=[str(b) for b in INVALID])
def test_invalid_simulation_parameters(pbf, bad):
    """RejectsInvalidSimulationParameters (test/test_pbf_solver.cu:204-327)."""
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize(8, (0, 0, 0), (2, 2, 2), pbf.SimulationParams(**P(**bad)))


def test_invalid_colliders_and_strong_guarantee(pbf):
    """PropagatesInvalidColliderConfiguration + RejectsInvalid{Sphere,Box,Plane}*."""
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.set_spheres([((0, 0, 0), 0.0)])
    with pytest.raises(pbf.InvalidArgument):
        s.set_spheres([((math.nan, 0, 0), 1.0)])
    with pytest.raises(pbf.InvalidArgument):
        s.set_boxes([((0, 0, 0), (1, -1, 1))])
    with pytest.raises(pbf.InvalidArgument):
        s.set_boxes([((0, 0, 0), (1, math.inf, 1))])
    with pytest.raises(pbf.InvalidArgument):
        s.set_planes([((0, 0, 0), (0, 0, 0))])
    with pytest.raises(pbf.InvalidArgument):
        s.set_planes([((0, math.inf, 0), (0, 1, 0))])
    s.set_spheres([((0, 0, 0), 1.0)])
    s.set_spheres([])
    s.set_boxes([])
    s.set_planes([])


def test_stage_argument_checks(pbf):
    """Grid validation of SpatialGrid::initialize (test/test_spatial_grid.cu:190-330)."""
    assert pbf.grid_dims((-2, -4, 1), (4, 2, 7), 2.0) == (3, 3, 3)
    assert pbf.grid_dims((-1, 2, 0), (4.1, 7.9, 2.01), 2.0) == (3, 3, 2)
    with pytest.raises(pbf.InvalidArgument):
        pbf.grid_dims((0, 0, 0), (1, 1, 1), 0.0)
    with pytest.raises(pbf.InvalidArgument):
        pbf.grid_dims((0, 0, 0), (1, 1, 1), -0.5)
    with pytest.raises(pbf.InvalidArgument):
        pbf.grid_dims((math.nan, 0, 0), (1, 1, 1), 1.0)
    with pytest.raises(pbf.InvalidArgument):
        pbf.grid_dims((0, 0, 0), (1, 1, 1), math.nan)
    with pytest.raises(pbf.InvalidArgument):
        pbf.grid_dims((0, 0, 0), (0, 2, 2), 1.0)
    with pytest.raises(pbf.LengthError):
        pbf.grid_dims((0, 0, 0), (1e20, 2, 2), 1.0)
    with pytest.raises(pbf.LengthError):  # more cells than 32-bit keys address
        pbf.grid_dims((0, 0, 0), (70000, 70000, 2), 1.0)
