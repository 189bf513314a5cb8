"""Compact neighbour lists (pbf_initialize_compact).

Each rebuild counts every particle's neighbours, scans the counts into list
offsets and writes each list contiguously.  The lists hold the same
neighbours in the same order as the slot-major lists, so whole steps agree
bit for bit; memory follows the actual neighbour count.  This is the
capacity policy for scenes whose densest particles need far more slots than
the average one (count, scan, then compact lists).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(pbf, scene, frames, max_nb=256, cap=None):
    pos, vel, mn, mx, prm, col = scene
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm, max_neighbors=max_nb, list_capacity=cap)
    if col.get("spheres"):
        s.set_spheres(col["spheres"])
    if col.get("boxes"):
        s.set_boxes(col["boxes"])
    s.set_particles(pos, vel)
    s.run(frames)
    out = (s.copy_positions_to_host(), s.copy_velocities_to_host(), s.density_error(),
           s.kernels_per_frame())
    s.close()
    return out


def same(a, b):
    np.testing.assert_array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
    assert a[2] == b[2]


def test_compact_lists_match_slot_major_bit_for_bit(pbf, scenes):
    sc = scenes.dam_break_16k()  # XSPH and vorticity on
    fixed = run(pbf, sc, 10)
    compact = run(pbf, sc, 10, cap=len(sc[0]) * 64)
    same(fixed, compact)
    # Per rebuild: one count kernel and three scan kernels more.
    assert compact[3] == fixed[3] + 5 * 4


def test_compact_lists_with_colliders_and_substeps(pbf, scenes):
    sc = scenes.reference_benchmark(16384)  # box + sphere, 2 substeps
    same(run(pbf, sc, 6), run(pbf, sc, 6, cap=16384 * 64))


def test_compact_lists_on_an_imbalanced_scene(pbf, scenes):
    # Half a lattice column, half 16 Gaussian blobs: the blob cores hold
    # several times the lattice's neighbour count.
    sc = scenes.imbalanced_8m(n_total=1 << 20)
    n = len(sc[0])
    fixed = run(pbf, sc, 3, max_nb=512)
    compact = run(pbf, sc, 3, max_nb=512, cap=n * 96)  # 5.3x less list memory
    same(fixed, compact)


def test_compact_capacity_overflow_is_reported(pbf, scenes):
    pos, vel, mn, mx, prm, _ = scenes.dam_break_16k()
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm, list_capacity=len(pos) * 4)  # ~30 needed
    s.set_particles(pos, vel)
    with pytest.raises(pbf.NeighborOverflowError, match="compact list capacity"):
        s.step()
    s.close()


def test_compact_lists_keep_the_per_particle_limit(pbf, scenes):
    pos, vel, mn, mx, prm, _ = scenes.dam_break_16k()
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm, max_neighbors=8, list_capacity=len(pos) * 64)
    s.set_particles(pos, vel)
    with pytest.raises(pbf.NeighborOverflowError, match="exceeds solver capacity"):
        s.step()
    s.close()
