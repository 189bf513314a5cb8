"""Oracle checks on committed fixtures (CPU).

contraction_pairs.npz (tests/golden/gen_contraction_pairs.py) holds isolated
particle pairs whose neighbour decision depends on how dx*dx + dy*dy + dz*dz is
rounded.  The reference's compiled findNeighbors decides every pair like
fma(dz, dz, fma(dy, dy, dx*dx)) (measured on a GB300, see
test_gpu_reference_cuda.py); the oracle must decide identically.
"""

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_pairs():
    f = np.load(os.path.join(GOLDEN, "contraction_pairs.npz"))
    forms = [str(x) for x in f["forms"]]
    return f["positions"], f["decisions"], forms


def pair_decisions(find, pos):
    mn, mx, h = (0.0, 0.0, 0.0), (20.0, 20.0, 20.0), 0.1
    return find(pos, mn, mx, h)


def test_fixture_discriminates_rounding_orders():
    pos, dec, forms = load_pairs()
    ref = dec[:, forms.index("z(y(xx))")]
    for other in ("z(x(yy))", "nofma", "x(y(zz))"):
        assert (dec[:, forms.index(other)] != ref).sum() >= 100, other


def test_oracle_distance_rounding_matches_reference_kernel(orc):
    pos, dec, forms = load_pairs()
    mn, h = (0.0, 0.0, 0.0), 0.1
    st, dims = orc.grid_dims(mn, (20.0, 20.0, 20.0), h)
    assert st == 0
    sk, si, cs, ce = orc.grid_build(pos, mn, h, dims)
    nb, cnt, ov = orc.find_neighbors(pos[si], cs, ce, dims, mn, h, h, 8, len(pos))
    counts = np.zeros(len(pos), np.int32)
    counts[si] = cnt
    assert (counts[0::2] == counts[1::2]).all()
    np.testing.assert_array_equal(counts[0::2].astype(bool), dec[:, forms.index("z(y(xx))")])
