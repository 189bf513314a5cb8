"""Two implementations behind one interface: the CPU oracle and the CUDA library.

The known-answer cases in cases.py run against both, so every reference test
scenario pins the oracle on the CPU and the CUDA kernels on the GPU.
"""

from __future__ import annotations

import numpy as np

from conftest import load_pkg


def flat(colliders, width):
    out = []
    for c in colliders:
        row = []
        for part in c:
            if isinstance(part, (tuple, list, np.ndarray)):
                row.extend(float(v) for v in part)
            else:
                row.append(float(part))
        out.append(row)
    return np.asarray(out, np.float32).reshape(-1, width)


class OracleBackend:
    name = "oracle"

    def __init__(self, precision=32):
        from oracle import oracle as O
        self.O = O
        self.precision = precision

    # -- solver -----------------------------------------------------------------
    class _Solver:
        def __init__(self, O, s):
            self.O = O
            self.s = s

        def set_particles(self, pos, vel):
            self.s.set_particles(pos, vel)

        def step(self):
            st = self.s.step()
            return {0: "ok", 3: "overflow", 4: "not_converged"}[st]

        def run(self, frames):
            for _ in range(frames):
                st = self.step()
                if st != "ok":
                    return st
            return "ok"

        def positions(self):
            return self.s.positions()

        def velocities(self):
            return self.s.velocities()

    def solver(self, params, capacity, mn, mx, spheres=(), boxes=(), planes=(), max_neighbors=256):
        s = self.O.OracleSolver(self.precision)
        s.initialize(capacity, mn, mx, params, max_neighbors)
        s.set_colliders(flat(spheres, 4), flat(boxes, 6), flat(planes, 6))
        return self._Solver(self.O, s)

    # -- stages -----------------------------------------------------------------
    def grid_build(self, pos, mn, mx, cell):
        st, dims = self.O.grid_dims(mn, mx, cell)
        assert st == 0
        return self.O.grid_build(pos, mn, cell, dims)

    def grid_dims(self, mn, mx, cell):
        st, dims = self.O.grid_dims(mn, mx, cell)
        assert st == 0
        return dims

    def find_neighbors(self, sorted_pos, cs, ce, dims, mn, cell, h, max_nb=256, stride=None):
        return self.O.find_neighbors(sorted_pos, cs, ce, dims, mn, cell, h, max_nb, stride)

    def lam(self, pos, nb, cnt, cap, stride, h, m, rho0, eps):
        return self.O.lam(pos, np.ascontiguousarray(nb, np.uint32),
                          np.ascontiguousarray(cnt, np.int32), cap, stride, h, m, rho0, eps)

    def delta(self, pos, nb, cnt, cap, lam, stride, h, m, rho0, k, n, dq):
        return self.O.delta(pos, np.ascontiguousarray(nb, np.uint32),
                            np.ascontiguousarray(cnt, np.int32), cap, lam, stride, h, m, rho0, k,
                            n, dq)

    def xsph(self, pos, nb, cnt, cap, v, stride, h, c):
        return self.O.xsph(pos, np.ascontiguousarray(nb, np.uint32),
                           np.ascontiguousarray(cnt, np.int32), cap, v, stride, h, c)

    def vorticity(self, pos, v, nb, cnt, cap, stride, h):
        return self.O.vorticity(pos, v, np.ascontiguousarray(nb, np.uint32),
                                np.ascontiguousarray(cnt, np.int32), cap, stride, h)

    def confinement(self, pos, nb, cnt, cap, om, v, stride, h, dt, eps):
        return self.O.confinement(pos, np.ascontiguousarray(nb, np.uint32),
                                  np.ascontiguousarray(cnt, np.int32), cap, om, v, stride, h, dt,
                                  eps)

    def collision_pass(self, pos, kind, cmin, cmax, r, spheres=(), boxes=(), planes=()):
        O = self.O
        if kind == 0:
            return O.solve_container(pos, cmin, cmax, r)
        if kind == 1:
            return O.solve_spheres(pos, flat(spheres, 4), r)
        if kind == 2:
            return O.solve_boxes(pos, flat(boxes, 6), r)
        return O.solve_planes(pos, flat(planes, 6), r)

    def collide(self, pos, cmin, cmax, r, spheres=(), boxes=(), planes=()):
        p, st = self.O.collide(pos, cmin, cmax, r, flat(spheres, 4), flat(boxes, 6),
                               flat(planes, 6))
        return p, ("ok" if st == 0 else "not_converged")

    def resolve(self, pos, vin, vel, cmin, cmax, r, e, fr, spheres=(), boxes=(), planes=()):
        return self.O.resolve_velocities(pos, vin, vel, cmin, cmax, r, e, fr, flat(spheres, 4),
                                         flat(boxes, 6), flat(planes, 6))


class CudaBackend:
    name = "cuda"

    def __init__(self):
        self.pbf = load_pkg()

    class _Solver:
        def __init__(self, pbf, s):
            self.pbf = pbf
            self.s = s

        def set_particles(self, pos, vel):
            self.s.set_particles(pos, vel)

        def step(self):
            try:
                self.s.step()
            except self.pbf.NeighborOverflowError:
                return "overflow"
            except self.pbf.SolverRuntimeError as e:
                if "converge" in str(e):
                    return "not_converged"
                raise
            return "ok"

        def run(self, frames):
            try:
                self.s.run(frames)
            except self.pbf.NeighborOverflowError:
                return "overflow"
            except self.pbf.SolverRuntimeError as e:
                if "converge" in str(e):
                    return "not_converged"
                raise
            return "ok"

        def positions(self):
            return self.s.copy_positions_to_host()

        def velocities(self):
            return self.s.copy_velocities_to_host()

    def solver(self, params, capacity, mn, mx, spheres=(), boxes=(), planes=(), max_neighbors=256):
        s = self.pbf.PBFSolver()
        s.initialize(capacity, mn, mx, self.pbf.SimulationParams(**params), max_neighbors)
        if len(spheres):
            s.set_spheres(spheres)
        if len(boxes):
            s.set_boxes(boxes)
        if len(planes):
            s.set_planes(planes)
        return self._Solver(self.pbf, s)

    def grid_build(self, pos, mn, mx, cell):
        return self.pbf.grid_build(pos, mn, mx, cell)

    def grid_dims(self, mn, mx, cell):
        return self.pbf.grid_dims(mn, mx, cell)

    def find_neighbors(self, sorted_pos, cs, ce, dims, mn, cell, h, max_nb=256, stride=None):
        return self.pbf.find_neighbors(sorted_pos, cs, ce, dims, mn, cell, h, max_nb, stride)

    def lam(self, pos, nb, cnt, cap, stride, h, m, rho0, eps):
        return self.pbf.compute_lambda(pos, nb, cnt, cap, stride, h, m, rho0, eps)

    def delta(self, pos, nb, cnt, cap, lam, stride, h, m, rho0, k, n, dq):
        return self.pbf.compute_delta(pos, nb, cnt, cap, lam, stride, h, m, rho0, k, n, dq)

    def xsph(self, pos, nb, cnt, cap, v, stride, h, c):
        return self.pbf.xsph(pos, nb, cnt, cap, v, stride, h, c)

    def vorticity(self, pos, v, nb, cnt, cap, stride, h):
        return self.pbf.vorticity(pos, v, nb, cnt, cap, stride, h)

    def confinement(self, pos, nb, cnt, cap, om, v, stride, h, dt, eps):
        return self.pbf.confinement(pos, nb, cnt, cap, om, v, stride, h, dt, eps)

    def collision_pass(self, pos, kind, cmin, cmax, r, spheres=(), boxes=(), planes=()):
        return self.pbf.collision_pass(pos, kind, cmin, cmax, r, spheres, boxes, planes)

    def collide(self, pos, cmin, cmax, r, spheres=(), boxes=(), planes=()):
        try:
            return self.pbf.collide(pos, cmin, cmax, r, spheres, boxes, planes), "ok"
        except self.pbf.SolverRuntimeError:
            return None, "not_converged"

    def resolve(self, pos, vin, vel, cmin, cmax, r, e, fr, spheres=(), boxes=(), planes=()):
        return self.pbf.resolve_velocities(pos, vin, vel, cmin, cmax, r, e, fr, spheres, boxes,
                                           planes)
