"""Batched solver on the GPU.

Every scene of a batch must come out bit for bit as the same scene run alone
by a single-scene solver (itself bit-exact against the FP32 oracle): the
per-scene key offset keeps each scene's sort order, lists and sums unchanged.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_alone(pbf, per, steps):
    out = []
    for p, v, lo, hi, q in per:
        a = pbf.PBFSolver()
        a.initialize(len(p), lo, hi, q)
        a.set_particles(p, v)
        a.run(steps)
        out.append((a.copy_positions_to_host(), a.copy_velocities_to_host()))
        a.close()
    return out


@pytest.mark.parametrize("steps,lanes", [(1, 0), (6, 1), (6, 4), (6, 8)])
def test_batch_equals_each_scene_alone(pbf, scenes, steps, lanes):
    """Every scene of a batch steps bit for bit as it does alone (each scene
    alone walks split over 8 lanes, the default up to 20,480 particles; the
    batch of 28,716 particles with the default, 1, 4 or 8 lanes)."""
    sc, prm, pos, vel, per = scenes.batched_scenes(n_scenes=12, n_min=512, n_max=8192, seed=11)
    b = pbf.PBFSolver()
    b.initialize_batch(sc, prm)
    assert b.scene_count() == 12
    b.set_walk_lanes(lanes)
    b.set_particles(pos, vel)
    b.run(steps)
    bp, bv = b.copy_positions_to_host(), b.copy_velocities_to_host()
    off = 0
    for k, (ap, av) in enumerate(run_alone(pbf, per, steps)):
        n = len(ap)
        np.testing.assert_array_equal(bp[off:off + n], ap, err_msg="scene %d positions" % k)
        np.testing.assert_array_equal(bv[off:off + n], av, err_msg="scene %d velocities" % k)
        off += n
    assert off == len(bp)
    mean, mx = b.density_error()
    assert np.isfinite(mean) and mean < 0.5


def test_batched_configuration_every_scene_equals_its_solo_run(pbf, scenes):
    """The whole batched configuration: 256 scenes, counts log-uniform in
    [2,048, 65,536] (4.72 M particles), block sizes chosen by the autotuner
    as in the benchmark, 3 steps: every one of the 256 scenes bit for bit as
    the same scene stepped by its own single-scene solver."""
    sc, prm, pos, vel, per = scenes.batched_scenes()
    assert len(sc) == 256
    b = pbf.PBFSolver()
    b.initialize_batch(sc, prm)
    b.set_particles(pos, vel)
    b.autotune(1)  # times trial frames, then restores the initial state
    b.run(3)
    bp, bv = b.copy_positions_to_host(), b.copy_velocities_to_host()
    b.close()
    off = 0
    for k, (ap, av) in enumerate(run_alone(pbf, per, 3)):
        n = len(ap)
        np.testing.assert_array_equal(bp[off:off + n], ap, err_msg="scene %d positions" % k)
        np.testing.assert_array_equal(bv[off:off + n], av, err_msg="scene %d velocities" % k)
        off += n
    assert off == len(bp)


def test_batch_takes_exactly_all_particles(pbf, scenes):
    sc, prm, pos, vel, _ = scenes.batched_scenes(n_scenes=3, n_min=512, n_max=1024, seed=2)
    b = pbf.PBFSolver()
    b.initialize_batch(sc, prm)
    with pytest.raises(pbf.OutOfRange):
        b.set_particles(pos[:-1], vel[:-1])
    b.set_particles(pos, vel)
    b.step()
    # Back to one scene on the same handle.
    p, v, lo, hi, q = scenes.dam_break(8, 8, 8, (0.8, 0.8, 0.8))[:5]
    b.initialize(len(p), lo, hi, q)
    assert b.scene_count() == 0
    b.set_particles(p, v)
    b.step()
    assert np.isfinite(b.copy_positions_to_host()).all()


def test_batch_one_launch_per_stage(pbf, scenes):
    """A frame's kernel count does not grow with the number of scenes: one
    launch per stage covers them all.  8 and 20 scenes, 24,844 and 26,508
    particles: both sort in two passes of 25-26 tiles (the sort's launch
    count depends on the key count and bits, not on the scenes)."""
    counts = []
    for k, lo, hi in ((8, 2048, 4096), (20, 512, 2048)):
        sc, prm, pos, vel, _ = scenes.batched_scenes(n_scenes=k, n_min=lo, n_max=hi, seed=4)
        b = pbf.PBFSolver()
        b.initialize_batch(sc, prm)
        b.set_particles(pos, vel)
        b.step()
        counts.append(b.kernels_per_frame())
    assert counts[0] == counts[1]


def test_autotune_keeps_results_and_state(pbf, scenes):
    """pbf_autotune picks block sizes among 64/128/256/512 and a sort tile of
    1,024 or 4,096 keys, leaves the particle state where it was and changes
    no result bit."""
    pos, vel, mn, mx, prm, _ = scenes.dam_break_16k()
    a = pbf.PBFSolver()
    a.initialize(len(pos), mn, mx, prm)
    a.set_particles(pos, vel)
    a.run(3)
    x0, v0 = a.copy_positions_to_host(), a.copy_velocities_to_host()
    assert a.walk_lanes() == 8  # default up to 20,480 particles
    sizes = a.autotune(1)
    assert sizes.pop("sort_tile") in (1024, 4096)
    assert set(sizes.values()) <= {64, 128, 256, 512}
    assert a.walk_lanes() == 8  # the tuner leaves the lanes alone
    np.testing.assert_array_equal(a.copy_positions_to_host(), x0)
    np.testing.assert_array_equal(a.copy_velocities_to_host(), v0)
    a.run(4)
    b = pbf.PBFSolver()
    b.initialize(len(pos), mn, mx, prm)
    b.set_particles(x0, v0)
    b.run(4)
    np.testing.assert_array_equal(a.copy_positions_to_host(), b.copy_positions_to_host())
    np.testing.assert_array_equal(a.copy_velocities_to_host(), b.copy_velocities_to_host())


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_walk_lanes_change_no_result(pbf, scenes, orc, lanes):
    """Splitting each particle's stencil rows over 1, 2, 4 or 8 lanes writes
    the same lists: steps stay bit for bit those of the FP32 oracle."""
    pos, vel, mn, mx, prm, _ = scenes.dam_break_16k()
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm)
    s.set_walk_lanes(lanes)
    assert s.walk_lanes() == lanes
    s.set_particles(pos, vel)
    s.run(3)
    o = orc.OracleSolver(32)
    o.initialize(len(pos), mn, mx, prm.as_dict())
    o.set_particles(pos, vel)
    assert o.run(3) == 0
    assert np.array_equal(s.copy_positions_to_host().view(np.uint32), o.positions().view(np.uint32))
    assert np.array_equal(s.copy_velocities_to_host().view(np.uint32),
                          o.velocities().view(np.uint32))
