"""Regenerate contraction_pairs.npz: isolated particle pairs at distance ~h
whose neighbour decision (d2 <= h2, float32) depends on how
dx*dx + dy*dy + dz*dz is rounded.

Pairs sit on a coarse lattice (spacing 5h) in a 20^3 box with h = 0.1, so each
particle's only candidate is its partner.  For each pair the decision is
computed with exact rational arithmetic for nine rounding orders (fused
multiply-add chains and the unfused sum); only pairs on which the orders
disagree are kept.  `decisions[:, k]` is the decision under `forms[k]`.
The reference's compiled findNeighbors (src/pbf/neighbors.cu:73-74) agrees
with 'z(y(xx))' = fma(dz, dz, fma(dy, dy, dx*dx)) on every pair.
"""

import os
from fractions import Fraction as Fr

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def rnd32(v: Fr) -> np.float32:
    """Round an exact rational to the nearest float32 (ties to even)."""
    f = np.float32(float(v))
    cands = [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
    return min(cands, key=lambda x: (abs(Fr(float(x)) - v),
                                     int(np.frombuffer(np.float32(x).tobytes(), np.uint32)[0]) & 1))


def F(a):
    return Fr(float(a))


def fma32(a, b, c):
    return rnd32(F(a) * F(b) + F(c))


def mul32(a, b):
    return rnd32(F(a) * F(b))


def add32(a, b):
    return rnd32(F(a) + F(b))


FORMS = {
    "z(x(yy))": lambda x, y, z: fma32(z, z, fma32(x, x, mul32(y, y))),
    "z(y(xx))": lambda x, y, z: fma32(z, z, fma32(y, y, mul32(x, x))),
    "x(y(zz))": lambda x, y, z: fma32(x, x, fma32(y, y, mul32(z, z))),
    "x(z(yy))": lambda x, y, z: fma32(x, x, fma32(z, z, mul32(y, y))),
    "y(x(zz))": lambda x, y, z: fma32(y, y, fma32(x, x, mul32(z, z))),
    "y(z(xx))": lambda x, y, z: fma32(y, y, fma32(z, z, mul32(x, x))),
    "a(x(yy))+zz": lambda x, y, z: add32(fma32(x, x, mul32(y, y)), mul32(z, z)),
    "a(y(xx))+zz": lambda x, y, z: add32(fma32(y, y, mul32(x, x)), mul32(z, z)),
    "nofma": lambda x, y, z: add32(add32(mul32(x, x), mul32(y, y)), mul32(z, z)),
}


def main(n_pairs: int = 1500, seed: int = 123):
    rng = np.random.default_rng(seed)
    h2 = np.float32(0.1) * np.float32(0.1)
    first, second, decisions = [], [], []
    while len(first) < n_pairs:
        k = len(first)
        c = np.array([0.25 + 0.5 * (k % 38), 0.25 + 0.5 * ((k // 38) % 38),
                      0.25 + 0.5 * (k // (38 * 38))], np.float64)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        r = 0.1 * (1 + rng.uniform(-3e-7, 3e-7))
        a = c.astype(np.float32)
        b = (c + v * r).astype(np.float32)
        dx, dy, dz = np.float32(a[0] - b[0]), np.float32(a[1] - b[1]), np.float32(a[2] - b[2])
        dec = [bool(f(dx, dy, dz) <= h2) for f in FORMS.values()]
        if len(set(dec)) > 1:
            first.append(a)
            second.append(b)
            decisions.append(dec)
    pos = np.ones((2 * n_pairs, 4), np.float32)
    pos[0::2, :3] = np.array(first)
    pos[1::2, :3] = np.array(second)
    np.savez_compressed(os.path.join(HERE, "contraction_pairs.npz"), positions=pos,
                        decisions=np.array(decisions, bool), forms=np.array(list(FORMS)))


if __name__ == "__main__":
    main()
