"""The load-imbalanced configuration, scaled down, on the GPU.

imbalanced_262k: half a lattice column, half four Gaussian blobs whose cores
hold about 1,090 neighbours within h (the 8M configuration's blob density),
so a third of the particles exceed the reference's 256 list slots.

* With the stock 256 slots both this library and the reference's kernels
  report neighbour overflow (PBFSolver::step throws overflow_error,
  src/pbf/pbf_solver.cu:227-230).
* With 2,048 slots, and with compact lists, three steps are bit-exact against
  the FP32 oracle.
* Grid hashes, sort order, cell ranges and the 2,048-slot lists (slot order
  included) are bit-exact against the reference's own kernels.
"""

import numpy as np
import pytest

from test_gpu_parity import assert_bitwise

pytestmark = pytest.mark.gpu

STEPS = 3


@pytest.fixture(scope="module")
def scene(scenes):
    return scenes.imbalanced_262k()


@pytest.fixture(scope="module")
def oracle_run(orc, scene):
    pos, vel, mn, mx, prm, _ = scene
    o = orc.OracleSolver(32)
    o.initialize(len(pos), mn, mx, prm.as_dict(), 2048)
    o.set_particles(pos, vel)
    assert o.run(STEPS) == 0
    return o.positions(), o.velocities(), o.working()


def test_stock_capacity_overflows_like_the_reference(pbf, orc, scene):
    pos, vel, mn, mx, prm, _ = scene
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm)
    s.set_particles(pos, vel)
    with pytest.raises(pbf.NeighborOverflowError):
        s.step()
    if orc.ref_fatbins_available():
        r = orc.RefCudaSolver()
        r.initialize(len(pos), mn, mx, prm.as_dict())
        r.set_colliders()
        r.set_particles(pos, vel)
        assert r.step() == orc.REF_OVERFLOW
        r.close()


@pytest.mark.parametrize("lists", ["slot-major 2048", "compact"])
def test_steps_bit_exact_vs_fp32_oracle(pbf, scene, oracle_run, lists):
    pos, vel, mn, mx, prm, _ = scene
    s = pbf.PBFSolver()
    if lists == "compact":
        # Room for the mean list of about 210 entries with margin.
        s.initialize(len(pos), mn, mx, prm, 2048, list_capacity=400 * len(pos))
    else:
        s.initialize(len(pos), mn, mx, prm, 2048)
    s.set_particles(pos, vel)
    s.run(STEPS)
    op, ov, (owp, oid, ocnt) = oracle_run
    assert_bitwise(s.copy_positions_to_host(), op, "positions")
    assert_bitwise(s.copy_velocities_to_host(), ov, "velocities")
    wp, wid, wcnt = s.working_state()
    assert_bitwise(wid, oid, "working order")
    assert_bitwise(wcnt, ocnt, "neighbour counts")


def test_initial_lists_exceed_the_stock_capacity(pbf, scene):
    """The blob cores start with about 1,090 neighbours (the constraint then
    pushes them apart within a few steps)."""
    pos, _, mn, mx, prm, _ = scene
    h = prm.smoothingRadius
    sk, si, cs, ce = pbf.grid_build(pos, mn, mx, h)
    _, cnt, ov = pbf.find_neighbors(pos[si], cs, ce, pbf.grid_dims(mn, mx, h), mn, h, h, 2048,
                                    len(pos))
    assert not ov
    assert 1000 < cnt.max() <= 2048 and (cnt > 256).sum() > len(pos) // 5


def test_grid_and_lists_bit_exact_vs_reference_kernels(pbf, orc, scene):
    if not orc.ref_fatbins_available():
        pytest.skip("reference fatbins not built (oracle/_ref)")
    pos, _, mn, mx, prm, _ = scene
    h = prm.smoothingRadius
    r = orc.RefCudaSolver()
    r.initialize(len(pos), mn, mx, prm.as_dict(), 2048)
    want = r.grid_build(pos)
    got = pbf.grid_build(pos, mn, mx, h)
    for g, w, what in zip(got, want, ("keys", "indices", "cellStart", "cellEnd")):
        np.testing.assert_array_equal(g, w, err_msg=what)
    sp = pos[got[1]]
    rnb, rcnt, stride, rov = r.find_neighbors(sp)
    r.close()
    nb, cnt, ov = pbf.find_neighbors(sp, got[2], got[3], pbf.grid_dims(mn, mx, h), mn, h, h,
                                     2048, stride)
    assert not ov and not rov
    np.testing.assert_array_equal(cnt, rcnt)
    n = len(sp)
    for k in range(int(cnt.max())):
        used = cnt > k
        np.testing.assert_array_equal(nb[k * stride:k * stride + n][used],
                                      rnb[k * stride:k * stride + n][used],
                                      err_msg="slot %d" % k)
