"""Reverse-mode derivative of the PBF step on the GPU (pbf_adjoint_*).

The adjoint's directional derivatives of L = mean |x_T - target|^2 are
checked against the FP64 forward-mode gradient of the same steps
(oracle/pbf_diff_oracle.cpp, pinned on the CPU against the FP64 oracle
solver and its own central differences) and against FP64 central finite
differences, along random directions in x0 and v0 and along rest density and
XSPH strength, with and without vorticity confinement.  Tolerance: 1e-3
relative.

Over a few steps the FP32 and FP64 trajectories agree to rounding and both
references apply.  Over longer horizons the collapsing dam is chaotic (the
FP64 derivative itself grows by orders of magnitude and no longer matches
FP64 central differences), so the long-horizon check linearises the FP64
tangents about the GPU's own trajectory: the same derivative, evaluated on
the same states.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


VORTICITY = [0.0, 1e-4]


def scene(scenes, nx=16, ny=16, nz=8, seed=0, vorticity=0.0):
    box = (2 * nx * 0.05, ny * 0.05 * 1.5, 2 * nz * 0.05)
    pos, vel, mn, mx, prm, _ = scenes.dam_break(nx, ny, nz, box, seed=seed)
    prm.vorticityStrength = vorticity
    prm.xsphViscosity = 2e-5
    rng = np.random.default_rng(seed + 1)
    target = pos[:, :3].astype(np.float64) + np.array([0.3, 0.0, 0.0])
    target += rng.normal(0.0, 0.01 * 0.1, target.shape)
    return pos, vel, mn, mx, prm, target


def loss_grad(x, target):
    n = len(target)
    d = x[:, :3].astype(np.float64) - target
    g = np.zeros((n, 4), np.float32)
    g[:, :3] = (2.0 / n) * d
    return float((d * d).sum() / n), g


def adjoint_grads(pbf, pos, vel, mn, mx, prm, target, steps, every):
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=every)
    x, v = a.forward(pos, vel, steps)
    L, gx = loss_grad(x, target)
    gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
    a.close()
    return x, L, gx0[:, :3].astype(np.float64), gv0[:, :3].astype(np.float64), gr, gc


@pytest.mark.parametrize("vorticity", VORTICITY)
def test_taped_forward_follows_the_solver(pbf, scenes, vorticity):
    pos, vel, mn, mx, prm, _ = scene(scenes, vorticity=vorticity)
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=3)
    s = pbf.PBFSolver()
    s.initialize(len(pos), mn, mx, prm)
    s.set_particles(pos, vel)
    # One step from particle-id order runs the solver's kernels on the same
    # data: bit for bit the solver's step.
    x, v = a.forward(pos, vel, 1)
    s.run(1)
    np.testing.assert_array_equal(x, s.copy_positions_to_host())
    np.testing.assert_array_equal(v, s.copy_velocities_to_host())
    # Later steps: the solver carries its sorted order from step to step and
    # the adjoint restarts each step from particle-id order, so particles of
    # equal cell key meet in another order (sums rounded differently).
    x, v = a.forward(pos, vel, 5)
    s.run(4)
    np.testing.assert_allclose(x, s.copy_positions_to_host(), atol=2e-5, rtol=0)
    np.testing.assert_allclose(v, s.copy_velocities_to_host(), atol=2e-3, rtol=0)


def test_forward_restarts_from_its_own_state(pbf, scenes):
    pos, vel, mn, mx, prm, _ = scene(scenes)
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=4)
    x7, v7 = a.forward(pos, vel, 7)
    x3, v3 = a.forward(pos, vel, 3)
    x, v = a.forward(x3, v3, 4)
    np.testing.assert_array_equal(x, x7)
    np.testing.assert_array_equal(v, v7)


def test_backward_repeats_bit_for_bit(pbf, scenes):
    # The first backward uses the last segment the forward recorded; the
    # second recomputes it from its checkpoint.
    pos, vel, mn, mx, prm, target = scene(scenes)
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=3)
    x, _ = a.forward(pos, vel, 7)
    _, gx = loss_grad(x, target)
    first = a.backward(gx, np.zeros_like(gx))
    second = a.backward(gx, np.zeros_like(gx))
    a.close()
    np.testing.assert_array_equal(first[0], second[0])
    np.testing.assert_array_equal(first[1], second[1])
    assert first[2] == second[2] and first[3] == second[3]


@pytest.mark.parametrize("vorticity", VORTICITY)
def test_adjoint_matches_fp64_forward_mode_and_finite_differences(pbf, scenes, orc, vorticity):
    pos, vel, mn, mx, prm, target = scene(scenes, vorticity=vorticity)
    steps, every = 6, 4  # two segments, the second shorter
    x, L, gx0, gv0, gr, gc = adjoint_grads(pbf, pos, vel, mn, mx, prm, target, steps, every)
    n = len(pos)
    rng = np.random.default_rng(11)
    dirs_v = rng.standard_normal((3, n, 3))
    dirs_x = rng.standard_normal((2, n, 3)) * 1e-2
    # Forward mode (FP64): 3 v0 directions, 2 x0 directions, rho0, c.
    k = 7
    tv = np.zeros((k, n, 3))
    tx = np.zeros((k, n, 3))
    tv[:3] = dirs_v
    tx[3:5] = dirs_x
    trho = np.zeros(k)
    tc = np.zeros(k)
    trho[5] = 1.0
    tc[6] = 1.0
    p = prm.as_dict()
    x64, v64, txo, _ = orc.diff_rollout(pos, vel, p, mn, mx, steps, tx0=tx, tv0=tv, trho=trho,
                                        tc=tc)
    np.testing.assert_allclose(x[:, :3], x64, atol=5e-5, rtol=0)
    d = (x64 - target) * (2.0 / n)
    jvp = np.array([(d * txo[q]).sum() for q in range(k)])
    adj = np.array([(gv0 * dirs_v[0]).sum(), (gv0 * dirs_v[1]).sum(), (gv0 * dirs_v[2]).sum(),
                    (gx0 * dirs_x[0]).sum(), (gx0 * dirs_x[1]).sum(), gr, gc])
    rel = np.abs(adj - jvp) / np.abs(jvp)
    assert (rel <= 1e-3).all(), (adj, jvp, rel)

    # FP64 central differences along the first v0 direction and rest density.
    def loss64(v0=vel, **phys):
        xx, _ = orc.diff_rollout(pos, v0, p, mn, mx, steps, **phys)
        return float(((xx - target) ** 2).sum() / n)

    # A small step: larger ones cross the container clamps' kinks.
    e = 2.0 ** -24
    vp, vm = vel.copy(), vel.copy()
    vp[:, :3] += (e * dirs_v[0]).astype(np.float32)
    vm[:, :3] -= (e * dirs_v[0]).astype(np.float32)
    dvf = (vp[:, :3].astype(np.float64) - vm[:, :3].astype(np.float64)) / (2 * e)
    fd_v = (loss64(v0=vp) - loss64(v0=vm)) / (2 * e)
    adj_v = (gv0 * dvf).sum()
    assert abs(adj_v - fd_v) <= 1e-3 * abs(fd_v), (adj_v, fd_v)
    # The rest density is stepped in double: the loss is strongly curved where
    # the confinement's |eta| is small, beyond float32-sized steps.
    r0 = float(p["restDensity"])
    hr = 1e-8 * r0
    fd_r = (loss64(rest_density=r0 + hr) - loss64(rest_density=r0 - hr)) / (2 * hr)
    assert abs(gr - fd_r) <= 1e-3 * abs(fd_r), (gr, fd_r)


def test_autograd_function(pbf, scenes):
    torch = pytest.importorskip("torch")
    import importlib
    ag = importlib.import_module("fluid_simulator_gb300.autograd")
    pos, vel, mn, mx, prm, target = scene(scenes, 8, 8, 4)
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=2)
    dev = torch.device("cuda", 0)
    x0 = torch.tensor(pos, device=dev)
    v0 = torch.tensor(vel, device=dev, requires_grad=True)
    rho = torch.tensor(float(prm.restDensity), dtype=torch.float64, requires_grad=True)
    c = torch.tensor(float(prm.xsphViscosity), dtype=torch.float64, requires_grad=True)
    x, v = ag.rollout(a, x0, v0, rho, c, 5)
    t = torch.tensor(target, device=dev, dtype=torch.float64)
    L = ((x[:, :3].double() - t) ** 2).sum() / len(pos)
    L.backward()
    x_np, L2, gx0, gv0, gr, gc = adjoint_grads(pbf, pos, vel, mn, mx, prm, target, 5, 2)
    np.testing.assert_allclose(v0.grad[:, :3].cpu().numpy(), gv0, rtol=1e-5, atol=1e-9)
    assert abs(rho.grad.item() - gr) <= 1e-6 * abs(gr)
    assert abs(c.grad.item() - gc) <= 1e-6 * abs(gc)


def test_adjoint_with_substeps_matches_fp64_forward_mode(pbf, scenes, orc):
    # Two substeps per step: each substep is one taped step of dt / 2.
    pos, vel, mn, mx, prm, target = scene(scenes, vorticity=1e-4)
    prm.substeps = 2
    steps, every = 4, 3  # two segments of 6 and 2 substeps
    x, L, gx0, gv0, gr, gc = adjoint_grads(pbf, pos, vel, mn, mx, prm, target, steps, every)
    n = len(pos)
    rng = np.random.default_rng(17)
    dirs = rng.standard_normal((2, n, 3))
    k = 4
    tv = np.zeros((k, n, 3))
    tv[:2] = dirs
    trho = np.array([0.0, 0.0, 1.0, 0.0])
    tc = np.array([0.0, 0.0, 0.0, 1.0])
    x64, _, txo, _ = orc.diff_rollout(pos, vel, prm.as_dict(), mn, mx, steps, tv0=tv,
                                      trho=trho, tc=tc)
    np.testing.assert_allclose(x[:, :3], x64, atol=5e-5, rtol=0)
    d = (x64 - target) * (2.0 / n)
    jvp = np.array([(d * txo[q]).sum() for q in range(k)])
    adj = np.array([(gv0 * dirs[0]).sum(), (gv0 * dirs[1]).sum(), gr, gc])
    rel = np.abs(adj - jvp) / np.abs(jvp)
    assert (rel <= 1e-3).all(), (adj, jvp, rel)


def gpu_states(a, pos, vel, steps):
    """(steps, 2, n, 4): x, v at the start of each step of the taped forward."""
    out = np.zeros((steps, 2, len(pos), 4), np.float32)
    x, v = pos, vel
    for t in range(steps):
        out[t, 0], out[t, 1] = x, v
        x, v = a.forward(x, v, 1)
    return out


@pytest.mark.parametrize("vorticity", VORTICITY)
def test_adjoint_matches_fp64_tangents_along_its_trajectory(pbf, scenes, orc, vorticity):
    pos, vel, mn, mx, prm, target = scene(scenes, vorticity=vorticity)
    steps, every = 20, 7  # three segments, the last shorter
    n = len(pos)
    a = pbf.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=every)
    states = gpu_states(a, pos, vel, steps)
    x, v = a.forward(pos, vel, steps)
    d = x[:, :3].astype(np.float64) - target
    gx = np.zeros((n, 4), np.float32)
    gx[:, :3] = (2.0 / n) * d
    gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
    rng = np.random.default_rng(13)
    dirs = rng.standard_normal((3, n, 3))
    k = 5
    tv = np.zeros((k, n, 3))
    tv[:3] = dirs
    trho = np.array([0, 0, 0, 1.0, 0])
    tc = np.array([0, 0, 0, 0, 1.0])
    _, _, txo, _ = orc.diff_rollout(pos, vel, prm.as_dict(), mn, mx, steps, tv0=tv, trho=trho,
                                    tc=tc, states=states)
    jvp = np.array([(d * (2.0 / n) * txo[q]).sum() for q in range(k)])
    g = gv0[:, :3].astype(np.float64)
    adj = np.array([(g * dirs[0]).sum(), (g * dirs[1]).sum(), (g * dirs[2]).sum(), gr, gc])
    rel = np.abs(adj - jvp) / np.abs(jvp)
    assert (rel <= 1e-3).all(), (adj, jvp, rel)


# Colliders grazing the 16x16x8 lattice (x, y in [0.025, 0.8], z in
# [0.025, 0.4]): a sphere and a box reaching into its top layers and a
# slightly tilted floor a few millimetres into its bottom layer, so most
# particles feel a projection or a contact while the step stays well
# conditioned (colliders deep in the fluid push particles out violently and
# make the derivatives grow by orders of magnitude).
_N = np.array([0.02, 1.0, 0.0]) / np.linalg.norm([0.02, 1.0, 0.0])
COLLIDERS = dict(spheres=[(0.2, 0.9, 0.2, 0.12)], boxes=[(0.6, 0.85, 0.2, 0.05, 0.06, 0.05)],
                 planes=[(0.4, 0.0, 0.2) + tuple(float(v) for v in _N)])


def with_colliders(obj):
    obj.set_spheres(COLLIDERS["spheres"])
    obj.set_boxes(COLLIDERS["boxes"])
    obj.set_planes(COLLIDERS["planes"])
    return obj


def check_gradient(adj, jvp, ndirs, tol=1e-3):
    """Random v0 directions: the whole-gradient relative error estimated
    from the projections (for Gaussian r, E[(e.r)^2] = |e|^2; a single random
    projection may nearly cancel).  Parameters: each relative error."""
    e = adj[:ndirs] - jvp[:ndirs]
    grad = np.sqrt((e ** 2).sum() / (jvp[:ndirs] ** 2).sum())
    par = np.abs(adj[ndirs:] - jvp[ndirs:]) / np.abs(jvp[ndirs:])
    assert grad <= tol and (par <= tol).all(), (adj, jvp, grad, par)


def test_colliders_taped_forward_follows_the_solver(pbf, scenes):
    pos, vel, mn, mx, prm, _ = scene(scenes, vorticity=1e-4)
    a = pbf.PBFAdjoint()
    a.initialize(len(pos), mn, mx, prm, max_neighbors=128, checkpoint_every=3)
    with_colliders(a)
    s = with_colliders(pbf.PBFSolver())
    s.initialize(len(pos), mn, mx, prm)
    s.set_particles(pos, vel)
    x, v = a.forward(pos, vel, 1)
    s.run(1)
    np.testing.assert_array_equal(x, s.copy_positions_to_host())
    np.testing.assert_array_equal(v, s.copy_velocities_to_host())


def test_colliders_adjoint_matches_fp64_forward_mode(pbf, scenes, orc):
    pos, vel, mn, mx, prm, target = scene(scenes, vorticity=1e-4)
    n = len(pos)
    steps = 6
    a = pbf.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=4)
    with_colliders(a)
    x, _ = a.forward(pos, vel, steps)
    L, gx = loss_grad(x, target)
    gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
    a.close()
    gv0 = gv0[:, :3].astype(np.float64)
    rng = np.random.default_rng(23)
    dirs = rng.standard_normal((4, n, 3))
    k = 6
    tv = np.zeros((k, n, 3))
    tv[:4] = dirs
    trho = np.array([0.0, 0.0, 0.0, 0.0, 1.0, 0.0])
    tc = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 1.0])
    x64, _, txo, _ = orc.diff_rollout(pos, vel, prm.as_dict(), mn, mx, steps, tv0=tv, trho=trho,
                                      tc=tc, **COLLIDERS)
    np.testing.assert_allclose(x[:, :3], x64, atol=5e-5, rtol=0)
    d = (x64 - target) * (2.0 / n)
    jvp = np.array([(d * txo[q]).sum() for q in range(k)])
    adj = np.array([(gv0 * dirs[q]).sum() for q in range(4)] + [gr, gc])
    check_gradient(adj, jvp, 4)


def test_colliders_adjoint_matches_fp64_tangents_along_its_trajectory(pbf, scenes, orc):
    pos, vel, mn, mx, prm, target = scene(scenes, vorticity=1e-4)
    steps, every = 12, 5
    n = len(pos)
    a = pbf.PBFAdjoint()
    a.initialize(n, mn, mx, prm, max_neighbors=128, checkpoint_every=every)
    with_colliders(a)
    states = gpu_states(a, pos, vel, steps)
    x, _ = a.forward(pos, vel, steps)
    d = x[:, :3].astype(np.float64) - target
    gx = np.zeros((n, 4), np.float32)
    gx[:, :3] = (2.0 / n) * d
    gx0, gv0, gr, gc = a.backward(gx, np.zeros_like(gx))
    rng = np.random.default_rng(29)
    dirs = rng.standard_normal((4, n, 3))
    k = 6
    tv = np.zeros((k, n, 3))
    tv[:4] = dirs
    trho = np.array([0, 0, 0, 0, 1.0, 0])
    tc = np.array([0, 0, 0, 0, 0, 1.0])
    _, _, txo, _ = orc.diff_rollout(pos, vel, prm.as_dict(), mn, mx, steps, tv0=tv, trho=trho,
                                    tc=tc, states=states, **COLLIDERS)
    jvp = np.array([(d * (2.0 / n) * txo[q]).sum() for q in range(k)])
    g = gv0[:, :3].astype(np.float64)
    adj = np.array([(g * dirs[q]).sum() for q in range(4)] + [gr, gc])
    check_gradient(adj, jvp, 4)
