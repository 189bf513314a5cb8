"""The grid build's stable sort at the sizes where its implementation changes.

Up to 16,384 keys one thread-block cluster of 8 CTAs (2,048 keys each) sorts
in a single launch; above, tiles of 1,024 keys sort in passes of 2-3
launches.  At every boundary -- one key, one CTA's slice, a slice and one,
the last cluster size and one past it -- and with keys from 1-bit to 17-bit
grids and heavy duplication (thousands of particles in one cell), sorted
keys, permutation and cell ranges equal the oracle's stable counting sort
bit for bit.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = (1, 2, 31, 2047, 2048, 2049, 4096, 8191, 16383, 16384, 16385, 40000)


def _positions(n, extent, rng, clumped):
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.0, extent, (n, 3)).astype(np.float32)
    if clumped:
        # Half the particles in one cell: long runs of equal keys.
        pos[: n // 2, :3] = np.float32(0.05)
    return pos


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("extent,clumped", [(0.35, False), (2.55, False), (5.0, True)])
def test_grid_build_matches_oracle(pbf, orc, n, extent, clumped):
    rng = np.random.default_rng(n * 7 + int(extent * 100))
    mn, mx, cell = (0.0, 0.0, 0.0), (extent, extent, extent), 0.1
    pos = _positions(n, extent, rng, clumped)
    got = pbf.grid_build(pos, mn, mx, cell)
    st, dims = orc.grid_dims(mn, mx, cell)
    assert st == 0
    want = orc.grid_build(pos, mn, cell, dims)
    for g, w, name in zip(got, want, ("sorted keys", "permutation", "cell start", "cell end")):
        np.testing.assert_array_equal(np.asarray(g).view(np.uint32), np.asarray(w).view(np.uint32),
                                      err_msg=name)
