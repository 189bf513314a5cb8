"""Known-answer cases restating the reference's own tests.

Each case takes a backend (backends.OracleBackend or backends.CudaBackend) and
asserts the result the reference's test asserts, with the reference's
tolerance.  The docstring names the reference test it follows.
"""

from __future__ import annotations

import math
import os

import numpy as np

from conftest import (SOLVER_MAX, SOLVER_MIN, collision_params, f4, pair_density, self_density,
                      valid_params)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PI = 3.14159265358979323846


def near(a, b, tol):
    np.testing.assert_allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=0,
                               atol=tol)


# ---------------------------------------------------------------------------
# numpy restatements used as independent expected values
# ---------------------------------------------------------------------------

def np_keys(pos, mn, cell, dims):
    """referenceKey (test/test_spatial_grid.cu:77-103) in float32 numpy."""
    p = np.asarray(pos, np.float32)[:, :3]
    c = np.floor((p - np.asarray(mn, np.float32)) / np.float32(cell))
    c = np.nan_to_num(c, nan=0.0)
    c = np.clip(c, -2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64)
    c = np.clip(c, 0, np.asarray(dims) - 1)
    k = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    return (k & 0xFFFFFFFF).astype(np.uint32)


def np_build(pos, mn, cell, dims):
    """buildReference (test/test_spatial_grid.cu:105-138): stable sort + ranges."""
    keys = np_keys(pos, mn, cell, dims)
    idx = np.argsort(keys, kind="stable").astype(np.uint32)
    sk = keys[idx]
    cells = dims[0] * dims[1] * dims[2]
    cs = np.full(cells, -1, np.int32)
    ce = np.full(cells, -1, np.int32)
    n = len(sk)
    for i in range(n):
        k = sk[i]
        if i == 0 or sk[i - 1] != k:
            cs[k] = i
        if i == n - 1 or sk[i + 1] != k:
            ce[k] = i + 1
    return sk, idx, cs, ce


def np_brute(pos, h):
    """bruteForce (test/test_neighbors.cu:114-136), float32 differences."""
    p = np.asarray(pos, np.float32)[:, :3]
    d = p[:, None, :] - p[None, :, :]
    d2 = (d * d).sum(-1, dtype=np.float32)
    h2 = np.float32(h) * np.float32(h)
    out = []
    for i in range(len(p)):
        js = np.nonzero(d2[i] <= h2)[0]
        out.append(sorted(int(j) for j in js if j != i))
    return out


def run_search(B, positions, h, cell=1.0, max_nb=256, mn=(0, 0, 0), mx=(5, 5, 5)):
    """runNeighborSearch (test/test_neighbors.cu:24-112): grid, host sort, search,
    lists mapped back to original ids."""
    pos = f4(*positions) if not isinstance(positions, np.ndarray) else positions
    sk, perm, cs, ce = B.grid_build(pos, mn, mx, cell)
    dims = B.grid_dims(mn, mx, cell)
    sp = pos[perm]
    n = len(pos)
    nb, cnt, ov = B.find_neighbors(sp, cs, ce, dims, mn, cell, h, max_nb, n)
    counts = np.zeros(n, np.int64)
    lists = [None] * n
    for s in range(n):
        o = perm[s]
        counts[o] = cnt[s]
        k = min(cnt[s], max_nb)
        lists[o] = sorted(int(perm[nb[j * n + s]]) for j in range(k))
    return counts, lists, ov


# ---------------------------------------------------------------------------
# spatial grid (test/test_spatial_grid.cu)
# ---------------------------------------------------------------------------

GRID_MIN, GRID_MAX, GRID_CELL = (0.0, 0.0, 0.0), (4.0, 3.0, 2.0), 1.0


def case_grid_dims(B):
    """CalculatesExactGridDimensions / CeilsNonIntegralGridDimensions."""
    assert tuple(B.grid_dims((-2, -4, 1), (4, 2, 7), 2.0)) == (3, 3, 3)
    assert tuple(B.grid_dims((-1, 2, 0), (4.1, 7.9, 2.01), 2.0)) == (3, 3, 2)


def case_grid_small_builds(B):
    """BuildsSingleParticle / ParticlesInDifferentCells / SameCell / boundaries."""
    dims = B.grid_dims(GRID_MIN, GRID_MAX, GRID_CELL)
    sets = [
        f4([1.2, 0.4, 1.8, 1]),
        f4([0.2, 0.2, 0.2, 1], [1.2, 0.2, 0.2, 1], [2.2, 1.2, 0.2, 1], [3.2, 2.2, 1.2, 1]),
        f4([0.1, 0.1, 0.1, 1], [0.5, 0.5, 0.5, 1], [0.9, 0.9, 0.9, 1], [2.5, 0.5, 0.5, 1]),
        f4([0, 0, 0, 1], [4, 3, 2, 1], [3.999, 2.999, 1.999, 1], [-0.5, 5, 9, 1]),
    ]
    for pos in sets:
        got = B.grid_build(pos, GRID_MIN, GRID_MAX, GRID_CELL)
        exp = np_build(pos, GRID_MIN, GRID_CELL, dims)
        for g, e in zip(got, exp):
            np.testing.assert_array_equal(g, e)


def case_grid_empty_clears(B):
    """EmptyBuildClearsAllCellRanges (test/test_spatial_grid.cu:331)."""
    sk, si, cs, ce = B.grid_build(np.zeros((0, 4), np.float32), GRID_MIN, GRID_MAX, GRID_CELL)
    assert len(sk) == 0 and len(si) == 0
    assert (cs == -1).all() and (ce == -1).all() and len(cs) == 24


def case_grid_clamps_huge(B):
    """ClampsFinitePositionsBeyondIntegerCoordinateRange: keys {0, 23}, indices {1, 0}."""
    sk, si, _, _ = B.grid_build(f4([1e30, 1e30, 1e30, 1], [-1e30, -1e30, -1e30, 1]), GRID_MIN,
                                GRID_MAX, GRID_CELL)
    assert list(sk) == [0, 23]
    assert list(si) == [1, 0]


def case_grid_randomized_8193(B):
    """SpatialGridRandomizedTest: 8,193 particles from mt19937(0x5A17), bit-exact
    against the stable-sort reference (test/test_spatial_grid.cu:649-680)."""
    pos = np.fromfile(os.path.join(GOLDEN, "grid_8193.bin"), np.float32).reshape(-1, 4)
    mn, mx, cell = (-8.0, -5.0, -3.0), (9.0, 7.0, 6.0), 0.75
    dims = B.grid_dims(mn, mx, cell)
    got = B.grid_build(pos, mn, mx, cell)
    exp = np_build(pos, mn, cell, dims)
    for g, e in zip(got, exp):
        np.testing.assert_array_equal(g, e)
    assert np.all(np.diff(got[0].astype(np.int64)) >= 0)


# ---------------------------------------------------------------------------
# neighbour search (test/test_neighbors.cu)
# ---------------------------------------------------------------------------

def lattice(n, spacing):
    pts = []
    for z in range(n):
        for y in range(n):
            for x in range(n):
                pts.append([0.5 + x * spacing, 0.5 + y * spacing, 0.5 + z * spacing, 1.0])
    return np.asarray(pts, np.float32)


def case_neighbors_line(B):
    """FindsExpectedNeighborsAlongLine: counts 2,3,4,4,4,4,3,2."""
    pos = np.asarray([[0.5 + i * 0.5, 2, 2, 1] for i in range(8)], np.float32)
    counts, lists, _ = run_search(B, pos, 1.01)
    assert list(counts) == [2, 3, 4, 4, 4, 4, 3, 2]
    assert lists == np_brute(pos, 1.01)


def case_neighbors_lattices(B):
    """Three/FiveCubedLattice...: corner 7, edge 11, face 17, interior 26, symmetric."""
    for n, idx in ((3, (0, 1, 4, 13)), (5, (0, 2, 12, 62))):
        pos = lattice(n, 0.5)
        counts, lists, _ = run_search(B, pos, 0.9, cell=0.5)
        assert lists == np_brute(pos, 0.9)
        assert [counts[i] for i in idx] == [7, 11, 17, 26]
        for i, li in enumerate(lists):
            for j in li:
                assert i in lists[j]


def case_neighbors_misc(B):
    """Boundaries, sparse, dense cluster, identical positions, huge radius."""
    counts, _, _ = run_search(B, [[0.01, 0.01, 0.01, 1], [0.11, 0.01, 0.01, 1],
                                  [4.89, 4.99, 4.99, 1], [4.99, 4.99, 4.99, 1]], 0.15)
    assert list(counts) == [1, 1, 1, 1]
    counts, _, _ = run_search(B, [[0.1, 0.1, 0.1, 1], [1.1, 3.7, 2.2, 1], [2.5, 0.8, 4.1, 1],
                                  [3.9, 2.4, 0.7, 1], [4.8, 4.8, 4.8, 1]], 0.2)
    assert list(counts) == [0] * 5
    dense = np.asarray([[2.0 + 0.001 * i, 2, 2, 1] for i in range(32)], np.float32)
    counts, _, _ = run_search(B, dense, 0.5)
    assert list(counts) == [31] * 32
    same = np.asarray([[2, 2, 2, 1]] * 4, np.float32)
    counts, lists, _ = run_search(B, same, 0.75)
    assert list(counts) == [3] * 4 and lists == np_brute(same, 0.75)
    far = np.asarray([[-0.1, 0, 0, 1], [1, 1, 1, 1], [5.1, 5.1, 5.1, 1]], np.float32)
    _, lists, _ = run_search(B, far, 1e10)
    assert lists == np_brute(far, 1e10)


def case_neighbors_nonfinite(B):
    """Non-finite and huge coordinates: NaN, +-inf (inf - inf is NaN) and
    +-1e30 never pass d2 <= h2; the finite cluster still finds itself."""
    inf, nan = np.inf, np.nan
    pos = np.asarray([[2.0, 2.0, 2.0, 1], [2.1, 2.0, 2.0, 1], [2.0, 2.2, 2.0, 1],
                      [2.0, 2.0, 2.3, 1], [nan, 2.0, 2.0, 1], [2.0, nan, 2.0, 1],
                      [inf, 2.0, 2.0, 1], [inf, 2.0, 2.0, 1], [2.0, 2.0, -inf, 1],
                      [-inf, -inf, -inf, 1], [1e30, 2.0, 2.0, 1], [2.0, 2.0, -1e30, 1],
                      [4.9, 4.9, inf, 1], [4.9, 4.9, inf, 1]], np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        exp = np_brute(pos, 0.5)
    counts, lists, ov = run_search(B, pos, 0.5)
    assert not ov
    assert lists == exp
    assert list(counts) == [len(e) for e in exp]
    assert list(counts[:4]) == [3, 3, 3, 3] and not any(counts[4:])


def case_neighbors_cross_boundaries(B):
    """AllSixDirectionsAndDiagonalAcrossCellBoundaries."""
    pos = np.asarray([[2.01, 2.01, 2.01, 1], [1.99, 2.01, 2.01, 1], [2.01, 1.99, 2.01, 1],
                      [2.01, 2.01, 1.99, 1], [1.99, 1.99, 1.99, 1], [5.01, 5.01, 5.01, 1],
                      [4.99, 4.99, 4.99, 1], [-0.01, -0.01, -0.01, 1], [0.01, 0.01, 0.01, 1]],
                     np.float32)
    _, lists, _ = run_search(B, pos, 0.1)
    assert lists == np_brute(pos, 0.1)


def case_neighbors_random_257(B):
    """FixedSeedRandomParticlesMatchBruteForce: mt19937(12345), h 0.85, cell 0.6."""
    pos = np.fromfile(os.path.join(GOLDEN, "neighbors_257.bin"), np.float32).reshape(-1, 4)
    _, lists, ov = run_search(B, pos, 0.85, cell=0.6)
    assert not ov
    assert lists == np_brute(pos, 0.85)


def case_neighbors_overflow(B):
    """ReportsMaximumNeighborOverflow: full counts 11 with capacity 8, flag set."""
    pos = np.asarray([[2, 2, 2, 1]] * 12, np.float32)
    counts, _, ov = run_search(B, pos, 0.75, 1.0, 8)
    assert list(counts) == [11] * 12
    assert ov


def case_neighbors_slot_major(B):
    """WritesSlotMajorNeighbors: stride 8, capacity 4, untouched slots stay."""
    pos = f4([3.1, 1, 1, 1], [0.1, 1, 1, 1], [3.3, 1, 1, 1], [0.3, 1, 1, 1], [0.5, 1, 1, 1])
    mn, mx = (0, 0, 0), (5, 5, 5)
    sk, perm, cs, ce = B.grid_build(pos, mn, mx, 1.0)
    dims = B.grid_dims(mn, mx, 1.0)
    sp = pos[perm]
    nb, cnt, _ = B.find_neighbors(sp, cs, ce, dims, mn, 1.0, 0.45, 4, 8)
    exp = np_brute(sp, 0.45)
    for i in range(5):
        assert cnt[i] == len(exp[i])
        assert sorted(int(nb[k * 8 + i]) for k in range(cnt[i])) == exp[i]
    for i in range(5, 8):
        assert all(nb[k * 8 + i] == 0xFFFFFFFF for k in range(4))


# ---------------------------------------------------------------------------
# constraint kernels (test/test_pbf_solver_kernels.cu, test/test_correctness.cu)
# ---------------------------------------------------------------------------

def case_lambda_partial_blocks(B):
    """ComputeLambdaAccumulatesDensityAndGradientsAcrossPartialBlocks."""
    n, cap = 513, 3
    pos = np.tile(np.float32([5, 5, 5, 9]), (n, 1))
    pos[:4] = [[0, 0, 0, 7], [0.5, 0.5, 0.25, -3], [0, 0.6, 0.8, 2], [0, 0, 1.25, -8]]
    nb = np.zeros(n * cap, np.uint32)
    nb[0], nb[n], nb[2 * n] = 1, 2, 3
    cnt = np.zeros(n, np.int32)
    cnt[0] = cap
    lam = B.lam(pos, nb, cnt, cap, n, 1.0, 2.0, 3.0, 0.01)
    sw = 315.0 / (64.0 * PI)
    nw = sw * (1 - 0.5625) ** 3
    grad = 45.0 / PI * (1 - 0.75) ** 2
    gs = 2.0 / 3.0
    gsum = 2.0 * (gs * grad) ** 2
    near(lam[0], -(2.0 * (sw + nw) / 3.0 - 1) / (gsum + 0.01), 1e-5)
    near(lam[1], -(2.0 * sw / 3.0 - 1) / 0.01, 1e-5)
    near(lam[-1], -(2.0 * sw / 3.0 - 1) / 0.01, 1e-5)


def case_delta_w_zero(B):
    """ComputeDeltaPositionAppliesLambdaCorrectionAndLeavesWZero."""
    n, cap = 257, 3
    pos = np.tile(np.float32([4, 4, 4, 1]), (n, 1))
    pos[:4] = [[0, 0, 0, 3], [0.25, 0.5, 0.5, 5], [0, 0.6, 0.8, 7], [0, 0, 1.25, -1]]
    nb = np.zeros(n * cap, np.uint32)
    nb[0], nb[n], nb[2 * n] = 1, 2, 3
    cnt = np.zeros(n, np.int32)
    cnt[0] = cap
    lam = np.zeros(n, np.float32)
    lam[:3] = [2.0, -0.5, 3.0]
    d = B.delta(pos, nb, cnt, cap, lam, n, 1.0, 2.0, 4.0, 0.0, 0, 0.0)
    gm = 45.0 / PI * 0.25 ** 2
    ex = 2.0 / 4.0 * (2.0 - 0.5) * gm / 3.0
    near(d[0, :3], [ex, 2 * ex, 2 * ex], 1e-5)
    assert d[0, 3] == 0.0 and (d[1] == 0).all() and d[-1, 3] == 0.0


def case_scorr(B):
    """ArtificialPressureTest: -k at dq, paper formula at r = h/2, zero at and
    beyond h (exercised through delta p with a unit lambda sum of zero)."""
    # s_corr enters delta p as (lambda_i + lambda_j + s_corr) * grad W; with
    # zero lambdas the delta isolates s_corr * (m/rho0) * grad W.
    h, k, nexp, dq = 1.0, 0.001, 4, 0.3
    for r, expect in ((0.5, -k * ((1 - 0.25) / (1 - dq * dq)) ** (3 * nexp)), (1.0, 0.0),
                      (1.2, 0.0)):
        pos = f4([0, 0, 0, 1], [r, 0, 0, 1])
        nb = np.asarray([1, 0], np.uint32)
        cnt = np.asarray([1, 0], np.int32)
        d = B.delta(pos, nb, cnt, 1, np.zeros(2, np.float32), 2, h, 1.0, 1.0, k, nexp, dq)
        g = -45.0 / PI * (1 - r) ** 2 * (-1.0) if r < h else 0.0  # d/dx of spiky at -r
        near(d[0, 0], expect * g, 1e-7)


def case_correctness_double_oracle(B):
    """CoupledDensityLambdaAndCorrectionMatchDoublePrecisionOracle
    (test/test_correctness.cu:121-181): lambda to 2e-6 relative, delta to 2e-5."""
    pos = f4([0.49, 0.49, 0.49, 1], [0.51, 0.51, 0.51, 2], [0.25, 0.5, 0.5, 3],
             [0.75, 0.5, 0.5, 4], [0.5, 0.25, 0.5, 5], [0.5, 0.75, 0.5, 6], [0.5, 0.5, 0.25, 7],
             [0.5, 0.5, 0.75, 8], [0.49, 0.49, 0.49, 9], [3, 3, 3, 10])
    n, cap = len(pos), 16
    h, mass, rho0, eps, k, dq = 0.7, 0.4, 2.0, 0.03, 0.002, 0.2
    mn, mx, cell = (0, 0, 0), (4, 4, 4), 0.25
    sk, perm, cs, ce = B.grid_build(pos, mn, mx, cell)
    dims = B.grid_dims(mn, mx, cell)
    sp = pos[perm]
    nb_s, cnt_s, _ = B.find_neighbors(sp, cs, ce, dims, mn, cell, h, cap, n)
    # Map the lists back to the original order (checkNeighborhoods, :71-84).
    cnt = np.zeros(n, np.int32)
    nb = np.zeros(n * cap, np.uint32)
    for s in range(n):
        o = perm[s]
        cnt[o] = cnt_s[s]
        for kk in range(cnt_s[s]):
            nb[kk * n + o] = perm[nb_s[kk * n + s]]
    lam = B.lam(pos, nb, cnt, cap, n, h, mass, rho0, eps)
    d = B.delta(pos, nb, cnt, cap, lam, n, h, mass, rho0, k, 4, dq)
    P = pos[:, :3].astype(np.float64)

    def W(v):
        r2 = float(v @ v)
        return 0.0 if r2 >= h * h else 315.0 / (64 * PI * h ** 9) * (h * h - r2) ** 3

    def G(v):
        r = math.sqrt(float(v @ v))
        if r == 0 or r >= h:
            return np.zeros(3)
        return -45.0 / (PI * h ** 6) * (h - r) ** 2 / r * v

    ref = np.zeros(n)
    for i in range(n):
        rho, den, ctr = 0.0, eps, np.zeros(3)
        for j in range(n):
            dv = P[i] - P[j]
            rho += mass * W(dv)
            g = G(dv) * (mass / rho0)
            ctr += g
            den += g @ g
        den += ctr @ ctr
        ref[i] = -(rho / rho0 - 1) / den
        assert abs(lam[i] - ref[i]) <= 2e-6 * max(1.0, abs(ref[i]))
    wdq = W(np.array([dq, 0, 0]))
    for i in range(n):
        corr = np.zeros(3)
        for j in range(n):
            if i == j:
                continue
            dv = P[i] - P[j]
            sc = -k * (W(dv) / wdq) ** 4
            corr += mass / rho0 * (ref[i] + ref[j] + sc) * G(dv)
        near(d[i, :3], corr, 2e-5)
        assert d[i, 3] == 0.0


def case_xsph_closed_form(B):
    """AppliesPoly6WeightedJacobiVelocityCorrection (test/test_pbf_solver_kernels.cu:492-544)
    restated: v' = v + c sum (v_j - v_i) W."""
    pos = f4([0, 0, 0, 1], [0.5, 0, 0, 1], [0, 0.25, 0, 1])
    vel = f4([1, 0, 0, 5], [3, 1, 0, 6], [0, 0, 2, 7])
    nb = np.asarray([1, 0, 0, 2, 0, 0], np.uint32)  # slot-major, stride 3
    cnt = np.asarray([2, 1, 1], np.int32)
    h, c = 1.0, 0.5
    out = B.xsph(pos, nb, cnt, 2, vel, 3, h, c)

    def W(r):
        return 315.0 / (64 * PI) * (1 - r * r) ** 3

    exp0 = vel[0, :3] + c * ((vel[1, :3] - vel[0, :3]) * W(0.5) + (vel[2, :3] - vel[0, :3]) * W(0.25))
    near(out[0, :3], exp0, 1e-5)
    assert out[0, 3] == 5.0 and out[2, 3] == 7.0
    same = B.xsph(pos, nb, cnt, 2, vel, 3, h, 0.0)
    np.testing.assert_array_equal(same, vel)


def case_vorticity_reference(B):
    """VorticityConfinementTest.MatchesCpuReference (test/test_pbf_solver_kernels.cu:659-767)
    restated in float64: omega = sum grad_i W x (v_j - v_i); confinement
    v += dt eps (N x omega)."""
    rng = np.random.default_rng(7)
    n = 6
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 0.6, (n, 3))
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.uniform(-1, 1, (n, 3))
    vel[:, 3] = np.arange(n)
    h = 1.0
    cap = n
    nb = np.zeros(cap * n, np.uint32)
    cnt = np.zeros(n, np.int32)
    for i in range(n):
        js = [j for j in range(n) if j != i]
        cnt[i] = len(js)
        for k, j in enumerate(js):
            nb[k * n + i] = j
    om = B.vorticity(pos, vel, nb, cnt, cap, n, h)
    P = pos[:, :3].astype(np.float64)
    V = vel[:, :3].astype(np.float64)

    def G(v):
        r = math.sqrt(float(v @ v))
        if r == 0 or r >= h:
            return np.zeros(3)
        return -45.0 / (PI * h ** 6) * (h - r) ** 2 / r * v

    ref = np.zeros((n, 3))
    for i in range(n):
        for j in range(n):
            if i != j:
                ref[i] += np.cross(G(P[i] - P[j]), V[j] - V[i])
    near(om[:, :3], ref, 1e-5 * max(1.0, np.abs(ref).max()))
    dt, eps = 0.01, 0.2
    out = B.confinement(pos, nb, cnt, cap, om, vel, n, h, dt, eps)
    wl = np.linalg.norm(ref, axis=1)
    for i in range(n):
        eta = sum(((wl[j] - wl[i]) * G(P[i] - P[j]) for j in range(n) if j != i), np.zeros(3))
        nn = eta / np.linalg.norm(eta) if np.linalg.norm(eta) > 1e-6 else np.zeros(3)
        exp = V[i] + dt * eps * np.cross(nn, ref[i])
        near(out[i, :3], exp, 1e-4)
        assert out[i, 3] == vel[i, 3]


# ---------------------------------------------------------------------------
# collisions (test/test_collision_kernels.cu, test/test_collision_system.cu)
# ---------------------------------------------------------------------------

BIG = ((-10.0, -10.0, -10.0), (10.0, 10.0, 10.0))


def case_container_kernel(B):
    """SolveContainerKernelTest: five walls, open top, interior unchanged."""
    box = ((0, 0, 0), (10, 10, 10))
    p, m = B.collision_pass(f4([-2, -3, -4, 1], [12, 15, 14, 2]), 0, *box, 1.0)
    near(p, f4([1, 1, 1, 1], [9, 15, 9, 2]), 1e-5)
    assert m
    p, m = B.collision_pass(f4([5, 5, 5, 3], [1, 1, 9, 4]), 0, *box, 1.0)
    near(p, f4([5, 5, 5, 3], [1, 1, 9, 4]), 1e-5)
    assert not m


def case_sphere_kernel(B):
    """SolveSpheresKernelTest: penetration, centre, contact, array order."""
    sp = [((1, 2, 3), 2.0)]
    p, _ = B.collision_pass(f4([2, 2, 3, 1], [1, 2, 3, 2]), 1, *BIG, 0.5, spheres=sp)
    near(p, f4([3.5, 2, 3, 1], [3.5, 2, 3, 2]), 1e-5)
    p, m = B.collision_pass(f4([1.5, 0, 0, 3], [2, 0, 0, 4]), 1, *BIG, 0.5,
                            spheres=[((0, 0, 0), 1.0)])
    near(p, f4([1.5, 0, 0, 3], [2, 0, 0, 4]), 1e-5)
    assert not m
    p, _ = B.collision_pass(f4([0, 0, 0, 7]), 1, *BIG, 0.5,
                            spheres=[((0, 0, 0), 1.0), ((2.5, 0, 0), 1.0)])
    near(p, f4([1, 0, 0, 7]), 1e-5)


def case_box_kernel(B):
    """SolveBoxesKernelTest: face/edge/corner, interior to nearest face, centre tie."""
    bx = [((0, 0, 0), (1, 1, 1))]
    p, _ = B.collision_pass(f4([1.2, 0, 0, 1], [1.2, 1.2, 0, 2], [1.2, 1.2, 1.2, 3]), 2, *BIG,
                            0.5, boxes=bx)
    near(p[0], [1.5, 0, 0, 1], 1e-5)
    near(p[1, :2], [1 + 0.5 / math.sqrt(2)] * 2, 1e-5)
    assert p[1, 2] == 0.0
    near(p[2, :3], [1 + 0.5 / math.sqrt(3)] * 3, 1e-5)
    p, _ = B.collision_pass(f4([0.8, 0, 0, 1], [-0.8, 0, 0, 2], [0, 0.8, 0, 3], [0, 0, -0.8, 4]),
                            2, *BIG, 0.5, boxes=bx)
    near(p, f4([1.5, 0, 0, 1], [-1.5, 0, 0, 2], [0, 1.5, 0, 3], [0, 0, -1.5, 4]), 1e-5)
    p, _ = B.collision_pass(f4([0, 0, 0, 9]), 2, *BIG, 0.5, boxes=bx)
    near(p, f4([1.5, 0, 0, 9]), 1e-5)
    p, m = B.collision_pass(f4([1.5, 0, 0, 1], [2, 2, 0, 2]), 2, *BIG, 0.5, boxes=bx)
    near(p, f4([1.5, 0, 0, 1], [2, 2, 0, 2]), 1e-5)
    assert not m


def case_plane_kernel(B):
    """SolvePlanesKernelTest: normalised normal, contact, zero normal ignored."""
    p, _ = B.collision_pass(f4([2, 1.2, 3, 1], [2, -4, 3, 2]), 3, *BIG, 0.5,
                            planes=[((0, 1, 0), (0, 2, 0))])
    near(p, f4([2, 1.5, 3, 1], [2, 1.5, 3, 2]), 1e-5)
    p, m = B.collision_pass(f4([0, 1.5, 0, 3], [0, 2, 0, 4]), 3, *BIG, 0.5,
                            planes=[((0, 1, 0), (0, 1, 0))])
    near(p, f4([0, 1.5, 0, 3], [0, 2, 0, 4]), 1e-5)
    assert not m
    p, _ = B.collision_pass(f4([0, 0, 3, 5]), 3, *BIG, 0.5,
                            planes=[((0, 0, 0), (0, 0, 0)), ((1, 0, 0), (1, 0, 0)),
                                    ((0, 2, 0), (0, 1, 0))])
    near(p, f4([1.5, 2.5, 3, 5]), 1e-5)


def case_resolve_velocities(B):
    """ResolveVelocitiesKernelTest: walls, open top, tolerance, colliders."""
    box = ((0, 0, 0), (10, 10, 10))
    pos = f4([0.5, 5, 5, 1], [9.5, 5, 5, 2], [5, 0.5, 5, 3], [5, 5, 0.5, 4], [5, 5, 9.5, 5],
             [5, 20, 5, 6])
    vel = f4([-2, 4, 0, 11], [2, 4, 0, 12], [4, -2, 0, 13], [4, 0, -2, 14], [4, 0, 2, 15],
             [1, 2, 3, 16])
    out = B.resolve(pos, vel, vel, *box, 0.5, 0.5, 0.25)
    near(out, f4([1, 3, 0, 11], [-1, 3, 0, 12], [3, 1, 0, 13], [3, 0, 1, 14], [3, 0, -1, 15],
                 [1, 2, 3, 16]), 1e-5)
    out = B.resolve(f4([0.50005, 5, 5, 1]), f4([-2, 0, 0, 2]), f4([-2, 0, 0, 2]), *box, 0.5, 0, 0)
    near(out, f4([0, 0, 0, 2]), 1e-5)
    inx, iny = f4([-2, 0, 0, 1]), f4([0, -2, 0, 2])
    out = B.resolve(f4([1.50005, 0, 0, 3]), inx, inx, *BIG, 0.5, 0, 0, spheres=[((0, 0, 0), 1.0)])
    near(out[0, 0], 0.0, 1e-5)
    out = B.resolve(f4([1.50005, 0, 0, 4]), inx, inx, *BIG, 0.5, 0, 0,
                    boxes=[((0, 0, 0), (1, 1, 1))])
    near(out[0, 0], 0.0, 1e-5)
    out = B.resolve(f4([0, 0.50005, 0, 5]), iny, iny, *BIG, 0.5, 0, 0,
                    planes=[((0, 0, 0), (0, 1, 0))])
    near(out[0, 1], 0.0, 1e-5)
    sv = f4([-2, 4, 0, 4], [2, 4, 0, 5], [-2, 4, 0, 6])
    out = B.resolve(f4([1.5, 0, 0, 1], [1.5, 0, 0, 2], [2, 0, 0, 3]), sv, sv, *BIG, 0.5, 0.5,
                    0.25, spheres=[((0, 0, 0), 1.0)])
    near(out, f4([1, 3, 0, 4], [2, 4, 0, 5], [-2, 4, 0, 6]), 1e-5)
    out = B.resolve(f4([1.5, 0, 0, 1]), f4([-2, 4, 0, 2]), f4([-2, 4, 0, 2]), *BIG, 0.5, 1.0, 1.0,
                    spheres=[((0, 0, 0), 1.0)])
    near(out, f4([2, 0, 0, 2]), 1e-5)
    edge = 1 + 0.5 / math.sqrt(2)
    bv = f4([-2, -2, 2, 4], [-2, 4, 0, 5], [-2, 4, 0, 6])
    out = B.resolve(f4([edge, edge, 0, 1], [0.8, 0, 0, 2], [3, 0, 0, 3]), bv, bv, *BIG, 0.5, 0.0,
                    0.5, boxes=[((0, 0, 0), (1, 1, 1))])
    near(out, f4([0, 0, 1, 4], [0, 2, 0, 5], [-2, 4, 0, 6]), 1e-5)
    out = B.resolve(f4([0, 1.5, 0, 1]), f4([4, -2, 0, 2]), f4([4, -2, 0, 2]), *BIG, 0.5, 0.5,
                    0.25, planes=[((0, 0, 0), (0, 0, 0)), ((0, 1, 0), (0, 2, 0))])
    near(out, f4([3, 1, 0, 2]), 1e-5)


def case_collision_system(B):
    """CollisionSystemTest: rounded contacts converge, impenetrable sphere,
    rounded box edge, non-convergence reported, combined colliders."""
    for i in range(1, 65):
        p, st = B.collide(f4([1.3 + i * 0.001, 2.2, -0.65, 1]), *BIG, 0.1,
                          spheres=[((1.3, 2.1, -0.7), 0.7)])
        assert st == "ok"
        x, y, z = float(p[0, 0]) - np.float32(1.3), float(p[0, 1]) - np.float32(2.1), \
            float(p[0, 2]) + np.float32(0.7)
        near(math.sqrt(x * x + y * y + z * z), 0.8, 2e-6)
    _, st = B.collide(f4([1.01, 1.03, 0, 1]), *BIG, 0.1, boxes=[((0, 0, 0), (1, 1, 1))])
    assert st == "ok"
    _, st = B.collide(f4([0.01, 0.02, 0.03, 1]), *BIG, 0.1, planes=[((0, 0, 0), (1, 2, 3))])
    assert st == "ok"
    p, _ = B.collide(f4([0.2, 0, 0, 1]), *BIG, 0.5, spheres=[((0, 0, 0), 1.0)])
    near(p[0, 0], 1.5, 1e-5)
    p, _ = B.collide(f4([1.1, 1.1, 0, 1]), *BIG, 0.5, boxes=[((0, 0, 0), (1, 1, 1))])
    near(math.hypot(p[0, 0] - 1, p[0, 1] - 1), 0.5, 1e-5)
    _, st = B.collide(f4([-1.6, 0, 0, 1]), (-2, -2, -2), (2, 2, 2), 0.25,
                      spheres=[((-1.5, 0, 0), 0.5)])
    assert st == "not_converged"
    p, _ = B.collide(f4([-5.2, 5, 0, 1], [1.2, 5, 0, 2], [5, 2.8, 0, 3]), *BIG, 0.5,
                     spheres=[((-5, 5, 0), 1.0)], boxes=[((0, 5, 0), (1, 1, 1))],
                     planes=[((0, 3, 0), (0, 1, 0))])
    near([p[0, 0], p[1, 0], p[2, 1]], [-6.5, 1.5, 3.5], 1e-5)


# ---------------------------------------------------------------------------
# whole solver (test/test_pbf_solver.cu)
# ---------------------------------------------------------------------------

def integrate_reference(p, v, dt, g, substeps):
    """integrateReference (test/test_pbf_solver.cu:70-83) in float32."""
    p = np.array(p, np.float32)
    v = np.array(v, np.float32)
    sdt = np.float32(dt) / np.float32(substeps)
    g = np.asarray(g, np.float32)
    for _ in range(substeps):
        v[:3] = v[:3] + g * sdt
        p[:3] = p[:3] + v[:3] * sdt
    return p, v


def case_solver_free_fall(B):
    """AdvancesSingleParticleWithGravity: dt 0.2, 4 substeps, 1e-5."""
    prm = valid_params()
    prm.update(dt=0.2, substeps=4, gravity=(1.0, -10.0, 2.0))
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    p0, v0 = [1, 5, 2, 17], [2, 3, -1, 23]
    s.set_particles(f4(p0), f4(v0))
    assert s.step() == "ok"
    ep, ev = integrate_reference(p0, v0, 0.2, (1, -10, 2), 4)
    near(s.positions()[0], ep, 1e-5)
    near(s.velocities()[0], ev, 1e-5)


def case_solver_two_particles(B):
    """SeparatesTwoNeighboringParticlesSymmetrically."""
    prm = valid_params()
    prm.update(dt=0.1, gravity=(0, 0, 0), solverIterations=3, substeps=1,
               restDensity=self_density(1.0, 1.0))
    s = B.solver(prm, 2, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([4.75, 5, 5, 3], [5.25, 5, 5, 4]), f4([0, 0, 0, 7], [0, 0, 0, 8]))
    assert s.step() == "ok"
    p, v = s.positions(), s.velocities()
    assert p[0, 0] < 4.75 and p[1, 0] > 5.25
    near(p[0, 0] + p[1, 0], 10.0, 1e-5)
    near(p[:, 1:3], 5.0, 1e-6)
    assert list(p[:, 3]) == [3, 4]
    assert v[0, 0] < 0 < v[1, 0]
    near(v[0, 0] + v[1, 0], 0.0, 1e-4)
    near(v[:, 1:3], 0.0, 1e-6)
    assert list(v[:, 3]) == [7, 8]


def case_solver_api_order(B):
    """SpatialReorderingPreservesOriginalApiOrder."""
    prm = valid_params()
    prm.update(gravity=(0, 0, 0), restDensity=self_density(1.0, 1.0))
    s = B.solver(prm, 5, SOLVER_MIN, SOLVER_MAX)
    pos = f4(*[[9 - 2 * i, 5, 5, 11 + i] for i in range(5)])
    vel = f4(*[[0.1 * (i + 1), 0, 0, 21 + i] for i in range(5)])
    s.set_particles(pos, vel)
    assert s.step() == "ok"
    p, v = s.positions(), s.velocities()
    for i in range(5):
        near(p[i], [pos[i, 0] + np.float32(0.1) * vel[i, 0], 5, 5, pos[i, 3]], 1e-5)
        near(v[i], vel[i], 1e-5)


def case_solver_run_semantics(B):
    """ExplicitFrameCountIsIndependentOfSolverIterations / NoArgumentRunAdvancesOneFrame."""
    prm = valid_params()
    prm.update(dt=0.1, gravity=(0, 0, 0), solverIterations=3, substeps=1)
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([1, 2, 3, 5]), f4([2, -1, 0.5, 6]))
    assert s.run(2) == "ok"
    near(s.positions()[0], [1 + 2 * 0.2, 2 - 0.2, 3 + 0.5 * 0.2, 5], 1e-5)
    near(s.velocities()[0], [2, -1, 0.5, 6], 1e-5)
    prm["solverIterations"] = 4
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([1, 2, 3, 4]), f4([2, -1, 0.5, 5]))
    assert s.run(1) == "ok"
    near(s.positions()[0], [1.2, 1.9, 3.05, 4.0], 1e-5)


def case_solver_1025_blocks(B):
    """AdvancesParticlesAcrossSeveralCudaBlocks: 1,025 particles, 2e-4."""
    n, w, sp = 1025, 11, 0.75
    prm = valid_params()
    prm.update(dt=0.02, smoothingRadius=0.5, particleMass=0.25,
               restDensity=self_density(0.25, 0.5), lambdaEpsilon=0.1, solverIterations=2,
               substeps=2, gravity=(0.5, -9.8, -0.25))
    s = B.solver(prm, n + 100, SOLVER_MIN, SOLVER_MAX)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    for i in range(n):
        x, y, z = i % w, (i // w) % w, i // (w * w)
        pos[i] = [0.25 + sp * x, 0.25 + sp * y, 0.25 + sp * z, 1.0 + i % 5]
        vel[i] = [0.1 + 0.00001 * x, 0.2 + 0.00001 * y, -0.3 + 0.00001 * z, 10.0 + i % 7]
    s.set_particles(pos, vel)
    assert s.step() == "ok"
    p, v = s.positions(), s.velocities()
    for i in range(n):
        ep, ev = integrate_reference(pos[i], vel[i], 0.02, (0.5, -9.8, -0.25), 2)
        near(p[i], ep, 2e-4)
        near(v[i], ev, 2e-4)
    assert np.isfinite(p).all() and np.isfinite(v).all()


def case_solver_collisions(B):
    """Restitution/friction and collider forwarding (test/test_pbf_solver.cu:115-133,
    665-706, 744-854)."""
    prm = collision_params()
    prm.update(gravity=(0, -9.8, 0), collisionFriction=0.25)
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([5, -1.75, 5, 1]), f4([2, 0, 0, 0]))
    assert s.step() == "ok"
    near(s.velocities()[0, :2], [1.5, 0.0], 1e-5)

    prm = collision_params()
    prm.update(particleRadius=0.5, collisionRestitution=0.5, collisionFriction=0.25)
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([-1.4, 5, 5, 7]), f4([-2, 4, 0, 8]))
    assert s.step() == "ok"
    near(s.positions()[0], [-1.5, 5.4, 5, 7], 1e-5)
    near(s.velocities()[0], [1, 3, 0, 8], 1e-5)

    prm = collision_params()
    prm.update(particleRadius=0.5, collisionRestitution=0.5)
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(f4([-1.5, 5, 5, 1]), f4([-2, 0, 0, 2]))
    assert s.step() == "ok"
    near(s.positions()[0, 0], -1.5, 1e-6)
    near(s.velocities()[0, 0], 1.0, 1e-6)

    prm = collision_params()
    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX, spheres=[((3, 5, 5), 0.5)])
    s.set_particles(f4([4, 5, 5, 1]), f4([-4, 0, 0, 2]))
    assert s.step() == "ok"
    near(s.positions()[0], [3.75, 5, 5, 1], 1e-5)
    near(s.velocities()[0], [0, 0, 0, 2], 1e-5)

    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX, boxes=[((3, 5, 5), (0.5, 0.5, 0.5))])
    s.set_particles(f4([4, 5, 5, 3]), f4([-4, 0, 0, 4]))
    assert s.step() == "ok"
    near(s.positions()[0], [3.75, 5, 5, 3], 1e-5)
    near(s.velocities()[0], [0, 0, 0, 4], 1e-5)

    s = B.solver(prm, 1, SOLVER_MIN, SOLVER_MAX, planes=[((0, 2, 0), (0, 2, 0))])
    s.set_particles(f4([5, 2.4, 5, 5]), f4([0, -3, 0, 6]))
    assert s.step() == "ok"
    near(s.positions()[0], [5, 2.25, 5, 5], 1e-5)
    near(s.velocities()[0], [0, 0, 0, 6], 1e-5)

    s = B.solver(prm, 3, SOLVER_MIN, SOLVER_MAX, spheres=[((2, 6, 2), 0.5)],
                 boxes=[((6, 6, 2), (0.5, 0.5, 0.5))], planes=[((0, 2, 0), (0, 1, 0))])
    s.set_particles(f4([3, 6, 2, 1], [7, 6, 2, 2], [10, 2.4, 2, 3]),
                    f4([-4, 0, 0, 4], [-4, 0, 0, 5], [0, -3, 0, 6]))
    assert s.step() == "ok"
    near(s.positions(), f4([2.75, 6, 2, 1], [6.75, 6, 2, 2], [10, 2.25, 2, 3]), 1e-5)
    near(s.velocities(), f4([0, 0, 0, 4], [0, 0, 0, 5], [0, 0, 0, 6]), 1e-5)


def case_solver_overflow(B):
    """RejectsNeighborOverflowBeforeConstraintSolve: 258 coincident particles."""
    prm = valid_params()
    prm.update(gravity=(0, 0, 0), particleRadius=0.01)
    s = B.solver(prm, 258, SOLVER_MIN, SOLVER_MAX)
    s.set_particles(np.tile(np.float32([5, 5, 5, 1]), (258, 1)), np.zeros((258, 4), np.float32))
    assert s.step() == "overflow"


def case_solver_xsph_after_collision(B):
    """XsphUsesNeighborsFromFinalCollisionCorrectedPositions."""
    prm = valid_params()
    prm.update(dt=0.1, gravity=(0, 0, 0), solverIterations=1, substeps=1, particleRadius=0.25,
               smoothingRadius=1.0, xsphViscosity=1.0)
    prm["restDensity"] = float(np.float32(self_density(1.0, 1.0)) +
                               np.float32(pair_density(1.0, 0.8, 1.0)))
    s = B.solver(prm, 2, SOLVER_MIN, SOLVER_MAX, spheres=[((5, 5, 5), 0.5)])
    s.set_particles(f4([4.6, 5, 5, 1], [5.4, 5, 5, 2]), f4([0, 0, 0, 3], [0, 0, 0, 4]))
    assert s.step() == "ok"
    p, v = s.positions(), s.velocities()
    near(p[:, 0], [4.25, 5.75], 1e-5)
    near(v[:, 0], [-3.5, 3.5], 1e-4)
    assert list(v[:, 3]) == [3, 4]


def case_solver_determinism(B):
    """FixedScenarioRepeatsExactly: two solvers, 10 frames, bit-identical."""
    prm = collision_params()
    prm.update(dt=0.01, substeps=2, solverIterations=3, xsphViscosity=0.03,
               vorticityStrength=0.02, scorrK=0.001, scorrN=4, scorrDeltaQ=0.15,
               gravity=(0, -1, 0))
    pos = f4([4.7, 6, 5, 1], [5.1, 6, 5, 2], [4.9, 6.35, 5, 3], [5.3, 6.35, 5, 4])
    vel = f4([0.1, 0, 0, 5], [-0.1, 0, 0, 6], [0, 0.1, 0, 7], [0, -0.1, 0, 8])
    outs = []
    for _ in range(2):
        s = B.solver(prm, 4, SOLVER_MIN, SOLVER_MAX)
        s.set_particles(pos, vel)
        assert s.run(10) == "ok"
        outs.append((s.positions(), s.velocities()))
    assert np.isfinite(outs[0][0]).all()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


ALL_CASES = [v for k, v in sorted(globals().items()) if k.startswith("case_")]
