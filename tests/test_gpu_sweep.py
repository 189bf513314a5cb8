"""Seeded sweep of scenes and parameters: CUDA steps bit-exact against the FP32 oracle.

Each case draws a lattice (shape, spacing, jitter, initial velocities, the
user payload in w), the solver parameters (iterations, substeps, dt, epsilon,
s_corr k / n / dq including the run-time exponent path n > 4, XSPH,
vorticity, restitution, friction, gravity), colliders (sphere, box, tilted
plane) and the neighbour-list layout (slot-major or compact), runs a few
frames on the GPU and in the oracle, and compares positions, velocities and
the working order bit for bit.  A case the oracle reports as failing must
fail on the GPU with the matching error.
"""

import numpy as np
import pytest

from backends import flat

pytestmark = pytest.mark.gpu

CASES = list(range(16))


def make_case(scenes, pbf, seed):
    rng = np.random.default_rng(1000 + seed)
    h = float(rng.choice([0.08, 0.1, 0.12]))
    sp = 0.5 * h
    r = 0.25 * h
    nx, ny, nz = (int(v) for v in rng.integers(6, 17, 3))
    pos = scenes.lattice(nx, ny, nz, sp, (r, r, r), float(rng.uniform(0.0, 0.05)) * h, seed)
    pos[:, 3] = rng.uniform(0.5, 2.0, len(pos)).astype(np.float32)  # payload, kept as is
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0.0, 0.3, (len(pos), 3)).astype(np.float32)
    vel[:, 3] = rng.uniform(-1.0, 1.0, len(pos)).astype(np.float32)
    box = (2.0 * nx * sp + 4 * r, 1.5 * ny * sp + 4 * r, 2.0 * nz * sp + 4 * r)
    rho0 = float(rng.choice([1000.0, 6378.0]))
    scorr_k = float(rng.choice([0.0, 1e-4, 1e-3]))
    prm = pbf.SimulationParams(
        dt=float(rng.choice([1.0 / 120.0, 1.0 / 240.0])),
        restDensity=rho0,
        particleMass=float(np.float32(rho0) * np.float32(sp) ** 3),
        particleRadius=r,
        collisionRestitution=float(rng.uniform(0.0, 0.5)),
        collisionFriction=float(rng.uniform(0.0, 0.3)),
        smoothingRadius=h,
        lambdaEpsilon=float(rng.choice([100.0, 600.0])),
        solverIterations=int(rng.choice([1, 2, 3, 5])),
        substeps=int(rng.choice([1, 2, 3])),
        gravity=(float(rng.uniform(-1.0, 1.0)), -9.8, float(rng.uniform(-1.0, 1.0))),
        scorrK=scorr_k,
        scorrN=int(rng.integers(1, 7)),
        scorrDeltaQ=float(rng.uniform(0.1, 0.3)) * h,
        xsphViscosity=float(rng.choice([0.0, 1e-5, 1e-4])),
        vorticityStrength=float(rng.choice([0.0, 1e-5, 1e-4])),
    )
    col = {}
    if rng.random() < 0.5:
        c = (box[0] * 0.7, box[1] * 0.2, box[2] * 0.5)
        col["spheres"] = [(c, float(min(box) * 0.15))]
    if rng.random() < 0.5:
        c = (box[0] * 0.8, box[1] * 0.15, box[2] * 0.3)
        col["boxes"] = [(c, (box[0] * 0.05, box[1] * 0.1, box[2] * 0.08))]
    if rng.random() < 0.5:
        nrm = np.array([rng.uniform(-0.3, 0.3), 1.0, rng.uniform(-0.3, 0.3)])
        nrm /= np.linalg.norm(nrm)
        col["planes"] = [((box[0] * 0.5, 0.3 * r, box[2] * 0.5), tuple(float(v) for v in nrm))]
    compact = bool(rng.random() < 0.5)
    return pos, vel, (0.0, 0.0, 0.0), box, prm, col, compact


@pytest.mark.parametrize("seed", CASES)
def test_random_case_bit_exact_vs_fp32_oracle(pbf, scenes, orc, seed):
    pos, vel, mn, mx, prm, col, compact = make_case(scenes, pbf, seed)
    n = len(pos)
    s = pbf.PBFSolver()
    s.initialize(n, mn, mx, prm, 256, list_capacity=n * 128 if compact else None)
    if col.get("spheres"):
        s.set_spheres(col["spheres"])
    if col.get("boxes"):
        s.set_boxes(col["boxes"])
    if col.get("planes"):
        s.set_planes(col["planes"])
    s.set_particles(pos, vel)
    o = orc.OracleSolver(32)
    o.initialize(n, mn, mx, prm.as_dict(), 256)
    o.set_colliders(flat(col.get("spheres", []), 4), flat(col.get("boxes", []), 6),
                    flat(col.get("planes", []), 6))
    o.set_particles(pos, vel)
    frames = 4
    st = o.run(frames)
    if st != 0:
        with pytest.raises(pbf.PBFError):
            s.run(frames)
        return
    s.run(frames)
    for got, want, what in ((s.copy_positions_to_host(), o.positions(), "positions"),
                            (s.copy_velocities_to_host(), o.velocities(), "velocities")):
        same = got.view(np.uint32) == want.view(np.uint32)
        assert same.all(), "%s differ at %d entries (case %d, compact=%s)" % (
            what, int((~same).sum()), seed, compact)
    _, wid, wcnt = s.working_state()
    _, oid, ocnt = o.working()
    np.testing.assert_array_equal(wid, oid)
    np.testing.assert_array_equal(wcnt, ocnt)
    s.close()
