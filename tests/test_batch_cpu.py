"""Batched-solver argument checks that need no GPU (pbf_batch_initialize
validates every scene before any CUDA call)."""

import math

import pytest

from conftest import valid_params


def scene(pbf, count=64, lo=(0, 0, 0), hi=(2, 2, 2), rho0=1000.0, mass=1.0, xsph=0.0):
    return pbf.Scene(count, lo, hi, rho0, mass, xsph)


def common(pbf, **kw):
    p = valid_params()
    p.update(kw)
    return pbf.SimulationParams(**p)


def test_batch_rejects_bad_scene_lists(pbf):
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize_batch([], common(pbf))
    with pytest.raises(pbf.InvalidArgument):  # a scene without particles
        s.initialize_batch([scene(pbf), scene(pbf, count=0)], common(pbf))
    with pytest.raises(pbf.InvalidArgument):  # XSPH on in one scene only
        s.initialize_batch([scene(pbf, xsph=0.0), scene(pbf, xsph=1e-5)], common(pbf))
    with pytest.raises(pbf.InvalidArgument):  # bad bounds
        s.initialize_batch([scene(pbf), scene(pbf, lo=(1, 0, 0), hi=(1, 2, 2))], common(pbf))
    with pytest.raises(pbf.InvalidArgument):  # container narrower than a diameter
        s.initialize_batch([scene(pbf, hi=(0.01, 2, 2))], common(pbf))
    with pytest.raises(pbf.LengthError):  # grid axis beyond int range
        s.initialize_batch([scene(pbf, hi=(1e20, 2, 2))], common(pbf, particleRadius=0.1))
    assert s.scene_count() == 0


@pytest.mark.parametrize("bad", [dict(rho0=0.0), dict(rho0=math.nan), dict(mass=-1.0),
                                 dict(mass=math.inf), dict(xsph=-1.0)])
def test_batch_rejects_bad_scene_parameters(pbf, bad):
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize_batch([scene(pbf), scene(pbf, **bad)], common(pbf))


def test_batch_rejects_bad_common_parameters(pbf):
    s = pbf.PBFSolver()
    with pytest.raises(pbf.InvalidArgument):
        s.initialize_batch([scene(pbf)], common(pbf, dt=0.0))
    with pytest.raises(pbf.InvalidArgument):
        s.initialize_batch([scene(pbf)], common(pbf), max_neighbors=0)


def test_batched_scene_generator(scenes):
    sc, prm, pos, vel, per = scenes.batched_scenes(n_scenes=8, n_min=512, n_max=4096, seed=3)
    assert len(sc) == 8 and pos.shape == vel.shape and pos.shape[0] == sum(s.count for s in sc)
    for s, (p, v, lo, hi, q) in zip(sc, per):
        assert len(p) == s.count and tuple(hi) == tuple(s.maxBounds)
        assert q.restDensity == s.restDensity and q.xsphViscosity == s.xsphViscosity
        assert 0.9 * 6378 <= s.restDensity <= 1.1 * 6378
