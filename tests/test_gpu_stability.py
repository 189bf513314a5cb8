"""The reference's long-run stability scenario on the GPU.

CorrectnessStabilityTest.DenseFluidWithSphereAndBoxFor1200Frames
(test/test_correctness.cu:183-267): a 10x10x10 block of fluid thrown at
(1, 0, 0.15) into a [0,3]x[0,3]x[0,2] container holding a sphere and a box,
1,200 frames of 2 substeps x 4 iterations.  Every frame: positions and
velocities finite, no penetration of the container, the sphere or the box
beyond 4e-6, nothing launched above y = 20, speed below 50.  Every 100 frames
and at the end the grid and the neighbour lists of the current positions are
checked against all pairs (checkNeighborhoods, :45-117).  At the end: contacts
with both colliders happened, mean height below 1, RMS speed below 1.

Beyond the reference's invariants, the trajectory is compared bit for bit
with the FP32 oracle every 100 frames.
"""

import numpy as np
import pytest

from cases import np_build

pytestmark = pytest.mark.gpu

SIDE, FRAMES, CAPACITY = 10, 1200, 256
TOL = np.float32(4e-6)
SPHERE = ((0.8, 0.45, 1.0), 0.22)
BOX = ((1.9, 0.35, 1.0), (0.22, 0.35, 0.4))
LO, HI = (0.0, 0.0, 0.0), (3.0, 3.0, 2.0)


def stability_params(pbf):
    """The scenario's SimulationParams (test/test_correctness.cu:185-202);
    unset fields are zero (value-initialised)."""
    f = np.float32
    return pbf.SimulationParams(
        dt=float(f(1.0) / f(60.0)), restDensity=1000.0,
        particleMass=float(f(1000) * f(0.12) * f(0.12) * f(0.12)), particleRadius=0.05,
        collisionRestitution=0.0, collisionFriction=0.03, smoothingRadius=0.24,
        lambdaEpsilon=100.0, solverIterations=4, substeps=2, gravity=(0.0, -9.81, 0.0),
        scorrK=0.0001, scorrN=4, scorrDeltaQ=0.072, xsphViscosity=0.00001,
        vorticityStrength=0.00001)


def stability_particles():
    """Lattice z -> y -> x, (0.35 + 0.12x, 1.1 + 0.12y, 0.4 + 0.12z) in float
    arithmetic; every velocity (1, 0, 0.15) (:208-211)."""
    f = np.float32
    pos = np.ones((SIDE ** 3, 4), np.float32)
    k = 0
    for z in range(SIDE):
        for y in range(SIDE):
            for x in range(SIDE):
                pos[k, 0] = f(0.35) + f(x) * f(0.12)
                pos[k, 1] = f(1.1) + f(y) * f(0.12)
                pos[k, 2] = f(0.4) + f(z) * f(0.12)
                k += 1
    vel = np.zeros_like(pos)
    vel[:, 0] = 1.0
    vel[:, 2] = np.float32(0.15)
    return pos, vel


def check_neighborhoods(pbf, orc, pos, h):
    """checkNeighborhoods: grid keys, permutation and ranges against the
    stable-sort restatement; lists against all pairs within h (as sets, with
    pairs at the rounding boundary of d2 <= h2 tolerated), and bit for bit in
    slot order against the FP32 oracle's findNeighbors."""
    n = len(pos)
    sk, si, cs, ce = pbf.grid_build(pos, LO, HI, h)
    dims = pbf.grid_dims(LO, HI, h)
    for got, want, what in zip((sk, si, cs, ce), np_build(pos, LO, h, dims),
                               ("keys", "indices", "cellStart", "cellEnd")):
        np.testing.assert_array_equal(got, want, err_msg=what)
    assert sorted(si.tolist()) == list(range(n))
    nb, cnt, ov = pbf.find_neighbors(pos[si], cs, ce, dims, LO, h, h, CAPACITY, n)
    assert not ov and cnt.max() <= CAPACITY
    onb, ocnt, _ = orc.find_neighbors(pos[si], cs, ce, dims, LO, h, h, CAPACITY, n)
    np.testing.assert_array_equal(cnt, ocnt)
    for k in range(int(cnt.max())):
        used = cnt > k
        np.testing.assert_array_equal(nb[k * n:(k + 1) * n][used], onb[k * n:(k + 1) * n][used])
    # All pairs, in the original order (float differences, x*x + y*y + z*z).
    p = pos[:, :3].astype(np.float32)
    d = p[:, None, :] - p[None, :, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    h2 = np.float32(h) * np.float32(h)
    near = np.abs(d2.astype(np.float64) - h2) <= 4 * np.spacing(h2)
    want = (d2 <= h2) & ~np.eye(n, dtype=bool)
    got = np.zeros((n, n), bool)
    for s in range(n):
        o = si[s]
        got[o, si[nb[np.arange(cnt[s]) * n + s]]] = True
    bad = (got != want) & ~near
    assert not bad.any(), "lists differ from all pairs at %s" % np.argwhere(bad)[:5]


def test_dense_fluid_with_sphere_and_box_1200_frames(pbf, orc):
    prm = stability_params(pbf)
    pos, vel = stability_particles()
    n = len(pos)
    s = pbf.PBFSolver()
    s.initialize(n, LO, HI, prm)
    s.set_spheres([SPHERE])
    s.set_boxes([BOX])
    s.set_particles(pos, vel)
    o = orc.OracleSolver(32)
    o.initialize(n, LO, HI, prm.as_dict())
    o.set_colliders([(*SPHERE[0], SPHERE[1])], [(*BOX[0], *BOX[1])], [])
    o.set_particles(pos, vel)

    r = np.float32(prm.particleRadius)
    c = np.array(SPHERE[0], np.float64)
    rad = np.float32(SPHERE[1])
    bc, be = np.array(BOX[0], np.float64), np.array(BOX[1], np.float64)
    peak = 0.0
    sphere_contacts = box_contacts = 0
    for frame in range(FRAMES):
        s.step()
        p = s.copy_positions_to_host()
        v = s.copy_velocities_to_host()
        assert np.isfinite(p[:, :3]).all() and np.isfinite(v[:, :3]).all(), frame
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        assert (x >= r - TOL).all() and (x <= np.float32(3) - r + TOL).all(), frame
        assert (y >= r - TOL).all() and (y < np.float32(20)).all(), frame
        assert (z >= r - TOL).all() and (z <= np.float32(2) - r + TOL).all(), frame
        p64 = p[:, :3].astype(np.float64)
        ds = np.sqrt(((p64 - c) ** 2).sum(1))
        assert (ds >= np.float64(rad + r - TOL)).all(), frame
        sphere_contacts += int((ds < np.float64(rad + r + np.float32(1e-4))).sum())
        q = np.maximum(0.0, np.abs(p64 - bc) - be)
        db = np.sqrt((q ** 2).sum(1))
        assert (db >= np.float64(r - TOL)).all(), frame
        box_contacts += int((db < np.float64(r + np.float32(1e-4))).sum())
        v2 = (v[:, :3].astype(np.float64) ** 2).sum(1)
        peak = max(peak, float(np.sqrt(v2.max())))
        assert (v2 < 50.0 * 50.0).all(), frame
        rms, height = float(np.sqrt(v2.sum() / n)), float(p64[:, 1].sum() / n)
        assert o.step() == 0
        if frame % 100 == 0 or frame == FRAMES - 1:
            check_neighborhoods(pbf, orc, p, prm.smoothingRadius)
            np.testing.assert_array_equal(p.view(np.uint32), o.positions().view(np.uint32),
                                          err_msg="positions vs FP32 oracle, frame %d" % frame)
            np.testing.assert_array_equal(v.view(np.uint32), o.velocities().view(np.uint32),
                                          err_msg="velocities vs FP32 oracle, frame %d" % frame)
    assert sphere_contacts > 0 and box_contacts > 0
    assert height < 1.0, height
    assert rms < 1.0, rms
    print("stability: particles=%d frames=%d peak_speed=%.3f final_rms_speed=%.4f "
          "final_mean_height=%.4f sphere_contacts=%d box_contacts=%d"
          % (n, FRAMES, peak, rms, height, sphere_contacts, box_contacts))
