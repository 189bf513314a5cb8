"""Seeded synthetic scenes for the PBF step (no dataset is involved).

Each scene returns ``(positions, velocities, min_bounds, max_bounds, params,
colliders)`` with (n, 4) float32 arrays.  Lattices are laid out x fastest,
then y, then z; w = 1.

* ``dam_break_16k``  -- 32x32x16 lattice, spacing 0.5h, jitter U(+-0.01h),
  box [0,1.6]x[0,1]x[0,0.8], origin at (r, r, r).
* ``dam_break_1m``   -- 128x128x64 lattice, same spacing and jitter,
  box [0,12.8]x[0,6.4]x[0,6.4] (the fluid fills the x<6.4, z<3.2 corner).
* ``imbalanced_8m``  -- half a dense lattice column, half 16 Gaussian blobs
  (sigma 4h, centres uniform), box 25.6x12.8x12.8.
* ``imbalanced_262k`` -- the same at 262,144 particles: half a lattice column,
  half 4 blobs of sigma 2h (the 8M blobs' core density), box 6.4x3.2x3.2.
* ``batched_scenes`` -- 256 independent dam breaks, particle counts
  log-uniform in [2,048, 65,536] (seed 7): a (2k, 2k, k) lattice per scene in
  a (4k, 2k, 2k) x spacing box, rest density x U(0.9, 1.1) with the mass
  scaled alike, XSPH c ~ U(0.005, 0.05) applied as c * m / rho0 (the
  reference's XSPH sum carries no m / rho factor, so an unscaled c >= 1e-4
  overshoots: c * sum W ~ c * rho0 / m).
* ``reference_benchmark`` -- the scene of the reference's benchmark
  (benchmark/pbf_benchmark.cu:20-114): 262,144 particles in 32 layers of
  128x64 at spacing 0.06 below y = 3.75, container [0,8.2]x[0,4]x[0,4.2], one
  box and one sphere collider, 2 substeps.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import SimulationParams

H = 0.1
SPACING = 0.5 * H
RADIUS = 0.025


def dam_break_params(rest_density: float = 6378.0, xsph: float = 1e-5) -> SimulationParams:
    """Dam-break parameters: h = 0.1, rho0 = 6378, eps = 600, 4 iterations,
    gravity -9.8, m = rho0 * spacing^3, dq = 0.2h, n = 4.

    One step() advances dt = 1/120 s (a 1/60 s frame as two steps), and the
    artificial-pressure, XSPH and vorticity strengths are the reference
    benchmark's tuned values (k = 1e-4, c = 1e-5, eps_v = 1e-5,
    benchmark/pbf_benchmark.cu:77-81).  The reference's kernels apply XSPH
    and vorticity without a mass/density factor, and with k = 0.1, c = 0.01,
    eps_v = 1e-4 or a single 1/60 s step its own update diverges on this
    lattice (velocities above 1e5 within 100 steps, neighbour counts past any
    capacity); with these values the density error stays near 5 %.
    """
    return SimulationParams(
        dt=1.0 / 120.0,
        restDensity=rest_density,
        particleMass=float(np.float32(rest_density) * np.float32(SPACING) ** 3),
        particleRadius=RADIUS,
        collisionRestitution=0.0,
        collisionFriction=0.03,
        smoothingRadius=H,
        lambdaEpsilon=600.0,
        solverIterations=4,
        substeps=1,
        gravity=(0.0, -9.8, 0.0),
        scorrK=1e-4,
        scorrN=4,
        scorrDeltaQ=0.2 * H,
        xsphViscosity=xsph,
        vorticityStrength=1e-5,
    )


def lattice(nx: int, ny: int, nz: int, spacing: float, origin, jitter: float, seed: int):
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float64) * spacing
    pts += np.asarray(origin, np.float64)
    if jitter:
        rng = np.random.default_rng(seed)
        pts += rng.uniform(-jitter, jitter, size=pts.shape)
    pos = np.ones((pts.shape[0], 4), np.float32)
    pos[:, :3] = pts.astype(np.float32)
    return pos


def dam_break(nx: int, ny: int, nz: int, box_max, seed: int = 0):
    pos = lattice(nx, ny, nz, SPACING, (RADIUS, RADIUS, RADIUS), 0.01 * H, seed)
    vel = np.zeros_like(pos)
    return pos, vel, (0.0, 0.0, 0.0), tuple(box_max), dam_break_params(), {}


def dam_break_16k(seed: int = 0):
    return dam_break(32, 32, 16, (1.6, 1.0, 0.8), seed)


def dam_break_1m(seed: int = 0):
    return dam_break(128, 128, 64, (12.8, 6.4, 6.4), seed)


def imbalanced_8m(seed: int = 0, n_total: int = 8_388_608):
    """Half a dense lattice column (corner), half 16 Gaussian blobs."""
    box = (25.6, 12.8, 12.8)
    half = n_total // 2
    # Column: 128 x 256 x 128 = 4,194,304 at spacing 0.5h from the corner.
    nx, nz = 128, 128
    ny = half // (nx * nz)
    col = lattice(nx, ny, nz, SPACING, (RADIUS, RADIUS, RADIUS), 0.01 * H, seed)
    rng = np.random.default_rng(seed + 1)
    centres = rng.uniform((2.0, 2.0, 2.0), (box[0] - 2.0, box[1] - 2.0, box[2] - 2.0), (16, 3))
    which = rng.integers(0, 16, n_total - col.shape[0])
    blob = centres[which] + rng.normal(0.0, 4 * H, (which.shape[0], 3))
    blob = np.clip(blob, RADIUS, np.asarray(box) - RADIUS)
    bl = np.ones((blob.shape[0], 4), np.float32)
    bl[:, :3] = blob.astype(np.float32)
    pos = np.concatenate([col, bl], axis=0)
    vel = np.zeros_like(pos)
    return pos, vel, (0.0, 0.0, 0.0), box, dam_break_params(), {}


def imbalanced_262k(seed: int = 0):
    """The imbalanced configuration scaled down to 262,144 particles with the
    same blob-core density: half a 64x32x64 lattice column in the corner,
    half 4 Gaussian blobs of sigma 2h (32,768 particles each, about 1,090
    neighbours within h at a blob's centre, as in the 8M scene's blobs),
    centres uniform in the inner part of a 6.4x3.2x3.2 box."""
    box = (6.4, 3.2, 3.2)
    col = lattice(64, 32, 64, SPACING, (RADIUS, RADIUS, RADIUS), 0.01 * H, seed)
    rng = np.random.default_rng(seed + 1)
    centres = rng.uniform((0.8, 0.8, 0.8), (box[0] - 0.8, box[1] - 0.8, box[2] - 0.8), (4, 3))
    which = np.repeat(np.arange(4), 32768)
    blob = centres[which] + rng.normal(0.0, 2 * H, (which.shape[0], 3))
    blob = np.clip(blob, RADIUS, np.asarray(box) - RADIUS)
    bl = np.ones((blob.shape[0], 4), np.float32)
    bl[:, :3] = blob.astype(np.float32)
    pos = np.concatenate([col, bl], axis=0)
    vel = np.zeros_like(pos)
    return pos, vel, (0.0, 0.0, 0.0), box, dam_break_params(), {}


def reference_benchmark_params() -> SimulationParams:
    """simulationParams() of benchmark/pbf_benchmark.cu:63-83."""
    spacing = np.float32(0.06)
    return SimulationParams(
        dt=1.0 / 60.0,
        restDensity=1000.0,
        particleMass=float(np.float32(1000.0) * spacing * spacing * spacing),
        particleRadius=0.025,
        collisionRestitution=0.0,
        collisionFriction=0.03,
        smoothingRadius=0.12,
        lambdaEpsilon=100.0,
        solverIterations=4,
        substeps=2,
        gravity=(0.0, -9.81, 0.0),
        scorrK=0.0001,
        scorrN=4,
        scorrDeltaQ=0.036,
        xsphViscosity=0.00001,
        vorticityStrength=0.00001,
    )


def reference_benchmark(n: int = 262_144):
    """createParticles of benchmark/pbf_benchmark.cu:85-114 (float32 arithmetic)."""
    px, pz = 128, 64
    if n % (px * pz):
        raise ValueError("particle count must contain whole 128x64 layers")
    layers = n // (px * pz)
    sp = np.float32(0.06)
    cmax = (8.2, 4.0, 4.2)
    width = np.float32(px - 1) * sp
    depth = np.float32(pz - 1) * sp
    sx = (np.float32(cmax[0]) - width) * np.float32(0.5)
    sz = (np.float32(cmax[2]) - depth) * np.float32(0.5)
    y, z, x = np.meshgrid(np.arange(layers), np.arange(pz), np.arange(px), indexing="ij")
    pos = np.ones((n, 4), np.float32)
    pos[:, 0] = sx + x.ravel().astype(np.float32) * sp
    pos[:, 1] = np.float32(3.75) - y.ravel().astype(np.float32) * sp
    pos[:, 2] = sz + z.ravel().astype(np.float32) * sp
    vel = np.zeros_like(pos)
    colliders = {
        "boxes": [((2.4, 0.675, 2.1), (0.65, 0.625, 0.75))],
        "spheres": [((5.7, 0.8, 2.1), 0.75)],
    }
    return pos, vel, (0.0, 0.0, 0.0), cmax, reference_benchmark_params(), colliders


SCENES = {
    "dam_break_16k": dam_break_16k,
    "dam_break_1m": dam_break_1m,
    "imbalanced_8m": imbalanced_8m,
    "imbalanced_262k": imbalanced_262k,
    "reference_benchmark": reference_benchmark,
}


def batched_scenes(n_scenes: int = 256, n_min: int = 2048, n_max: int = 65536, seed: int = 7):
    """Returns (scenes, common, positions, velocities, per_scene) where scenes
    is a list of ``Scene`` records, common the shared SimulationParams,
    positions / velocities the concatenation in scene order and per_scene a
    list of (positions, velocities, min_bounds, max_bounds, SimulationParams)
    for running each scene alone."""
    from . import Scene

    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_scenes))
    common = dam_break_params()
    scenes, per, P, V = [], [], [], []
    for s in range(n_scenes):
        k = max(2, int(round((targets[s] / 4.0) ** (1.0 / 3.0))))
        nx, ny, nz = 2 * k, 2 * k, k
        box = (2 * nx * SPACING, ny * SPACING, 2 * nz * SPACING)
        pos = lattice(nx, ny, nz, SPACING, (RADIUS, RADIUS, RADIUS), 0.01 * H, seed * 1000 + s)
        vel = np.zeros_like(pos)
        scale = float(rng.uniform(0.9, 1.1))
        rho0 = float(np.float32(common.restDensity * scale))
        mass = float(np.float32(rho0) * np.float32(SPACING) ** 3)
        c = float(rng.uniform(0.005, 0.05))
        xsph = float(np.float32(c * mass / rho0))
        scenes.append(Scene(len(pos), (0.0, 0.0, 0.0), box, rho0, mass, xsph))
        prm = dataclasses.replace(common, restDensity=rho0, particleMass=mass, xsphViscosity=xsph)
        per.append((pos, vel, (0.0, 0.0, 0.0), box, prm))
        P.append(pos)
        V.append(vel)
    return scenes, common, np.concatenate(P), np.concatenate(V), per
