"""This library against the reference's own CUDA kernels on the same GB300.

The reference kernels are its sources compiled by oracle/build_ref.py (Release
flags, sm_103a) and launched by oracle/ref_driver.cu with PBFSolver's host
sequence.  On identical inputs the cell hashes, the stable sort order, the
cell ranges and the neighbour lists (slot order included) must be identical;
whole steps agree within FP32 tolerance (the float arithmetic of the two
implementations is not the same sequence of operations).
Skipped when the reference fatbins were not built (no reference tree).
"""

import os

import numpy as np
import pytest

from backends import flat
from conftest import valid_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(orc):
    if not orc.ref_fatbins_available():
        pytest.skip("reference fatbins not built (oracle/_ref)")
    return orc


def ref_solver(orc, n, mn, mx, h):
    r = orc.RefCudaSolver()
    p = valid_params()
    p["smoothingRadius"] = h
    p["particleRadius"] = min(0.25 * h, 0.49 * (mx[0] - mn[0]))
    r.initialize(n, mn, mx, p)
    return r


def test_grid_bit_exact_on_golden_8193(pbf, ref):
    pos = np.fromfile(os.path.join(os.path.dirname(__file__), "golden", "grid_8193.bin"),
                      np.float32).reshape(-1, 4)
    mn, mx, cell = (-8.0, -5.0, -3.0), (9.0, 7.0, 6.0), 0.75
    r = ref_solver(ref, len(pos), mn, mx, cell)
    want = r.grid_build(pos)
    got = pbf.grid_build(pos, mn, mx, cell)
    for g, w, what in zip(got, want, ("keys", "indices", "cellStart", "cellEnd")):
        np.testing.assert_array_equal(g, w, err_msg=what)


@pytest.mark.parametrize("scene_name", ["dam_break_16k", "dam_break_1m"])
def test_grid_and_lists_bit_exact(pbf, scenes, ref, scene_name):
    pos, _, mn, mx, prm, _ = getattr(scenes, scene_name)()
    rng = np.random.default_rng(5)
    pos = pos.copy()
    pos[:, :3] += rng.normal(0, 0.01, (len(pos), 3)).astype(np.float32)
    h = prm.smoothingRadius
    r = ref_solver(ref, len(pos), mn, mx, h)
    want = r.grid_build(pos)
    got = pbf.grid_build(pos, mn, mx, h)
    for g, w, what in zip(got, want, ("keys", "indices", "cellStart", "cellEnd")):
        np.testing.assert_array_equal(g, w, err_msg=what)
    sp = pos[got[1]]
    rnb, rcnt, stride, rov = r.find_neighbors(sp)
    dims = pbf.grid_dims(mn, mx, h)
    nb, cnt, ov = pbf.find_neighbors(sp, got[2], got[3], dims, mn, h, h, 256, stride)
    assert not ov and not rov
    np.testing.assert_array_equal(cnt, rcnt)
    n = len(sp)
    for k in range(int(cnt.max())):
        used = cnt > k
        np.testing.assert_array_equal(nb[k * stride:k * stride + n][used],
                                      rnb[k * stride:k * stride + n][used],
                                      err_msg="slot %d" % k)


@pytest.mark.parametrize("steps,tol", [(1, 2e-5), (10, 1e-3)])
def test_steps_agree_with_reference_kernels(pbf, scenes, ref, steps, tol):
    """dam_break_16k and the reference benchmark's box + sphere scene."""
    for name, args in (("dam_break_16k", ()), ("reference_benchmark", (8192,))):
        pos, vel, mn, mx, prm, col = getattr(scenes, name)(*args)
        s = pbf.PBFSolver()
        s.initialize(len(pos), mn, mx, prm)
        if col.get("spheres"):
            s.set_spheres(col["spheres"])
        if col.get("boxes"):
            s.set_boxes(col["boxes"])
        s.set_particles(pos, vel)
        s.run(steps)
        r = ref.RefCudaSolver()
        r.initialize(len(pos), mn, mx, prm.as_dict())
        r.set_colliders(flat(col.get("spheres", []), 4), flat(col.get("boxes", []), 6), flat([], 6))
        r.set_particles(pos, vel)
        assert r.run(steps) == 0
        dp = np.abs(s.copy_positions_to_host()[:, :3] - r.positions()[:, :3])
        assert np.percentile(dp, 99.9) <= tol, (name, np.percentile(dp, 99.9))
        assert dp.max() <= 50 * tol, (name, dp.max())
        np.testing.assert_array_equal(s.copy_positions_to_host()[:, 3], r.positions()[:, 3])
