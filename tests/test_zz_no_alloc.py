"""The grid build that allocates nothing, checked against the allocating one.

pbf_grid_build_static_scratch serves callers that must not allocate device
memory while they run (real-time loops where cudaMalloc/cudaFree can block or
synchronise the device, programs whose device memory belongs to another
allocator).  It keeps its working memory in a fixed array inside the library,
so two calls in a row must each give exactly what pbf_grid_build gives, with
nothing left over from the previous call showing through.  Collected last
(file name) so a failure here never hides the rest of the suite.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f3(pbf, v):
    return pbf.Float3(float(v[0]), float(v[1]), float(v[2]))


def _call(L, pbf, d_pos, n, mn, mx, cell, d_sk, d_si, d_cs, d_ce, stream):
    return L.pbf_grid_build_static_scratch(
        C.c_void_p(d_pos.data_ptr()), n, _f3(pbf, mn), _f3(pbf, mx), cell,
        C.c_void_p(d_sk.data_ptr()), C.c_void_p(d_si.data_ptr()),
        C.c_void_p(d_cs.data_ptr()), C.c_void_p(d_ce.data_ptr()), stream)


def test_static_scratch_grid_build_matches_allocating_build_twice(pbf):
    torch = pytest.importorskip("torch")
    L = pbf.load()
    cap = L.pbf_static_scratch_capacity()
    assert cap == 262144
    mn, mx, cell = (-8.0, -5.0, -3.0), (9.0, 7.0, 6.0), 0.75
    dims = pbf.grid_dims(mn, mx, cell)
    cells = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(2024)
    side = torch.cuda.Stream()
    # Two calls in a row: a large set on the default stream, then a smaller
    # one on a caller's own stream, whose outputs would pick up stale entries
    # if the shared array leaked state between calls.
    for n, stream in ((cap, None), (4099, side)):
        pos = np.ones((n, 4), np.float32)
        pos[:, :3] = rng.uniform((-12, -9, -7), (13, 11, 10), (n, 3)).astype(np.float32)
        want = pbf.grid_build(pos, mn, mx, cell)  # allocating entry point, host arrays
        d_pos = torch.from_numpy(pos).cuda()
        d_sk = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_si = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_cs = torch.full((cells,), 123, dtype=torch.int32, device="cuda")
        d_ce = torch.full((cells,), 123, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        handle = None if stream is None else C.c_void_p(stream.cuda_stream)
        st = _call(L, pbf, d_pos, n, mn, mx, cell, d_sk, d_si, d_cs, d_ce, handle)
        assert st == 0, L.pbf_global_last_error()
        if stream is None:
            torch.cuda.synchronize()
        else:
            stream.synchronize()
        got = (d_sk.cpu().numpy().view(np.uint32), d_si.cpu().numpy().view(np.uint32),
               d_cs.cpu().numpy(), d_ce.cpu().numpy())
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)


def test_static_scratch_grid_build_allocates_no_device_memory(pbf):
    """After a first call (which may load the library's kernels on the
    device), a call leaves the device's free memory exactly as it was."""
    torch = pytest.importorskip("torch")
    L = pbf.load()
    n = 100000
    mn, mx, cell = (0.0, 0.0, 0.0), (4.0, 2.0, 2.0), 0.1
    dims = pbf.grid_dims(mn, mx, cell)
    cells = dims[0] * dims[1] * dims[2]
    pos = np.ones((n, 4), np.float32)
    pos[:, :3] = np.random.default_rng(7).uniform((0, 0, 0), (4, 2, 2), (n, 3))
    d_pos = torch.from_numpy(pos).cuda()
    d_sk = torch.empty((n,), dtype=torch.int32, device="cuda")
    d_si = torch.empty((n,), dtype=torch.int32, device="cuda")
    d_cs = torch.empty((cells,), dtype=torch.int32, device="cuda")
    d_ce = torch.empty((cells,), dtype=torch.int32, device="cuda")
    args = (L, pbf, d_pos, n, mn, mx, cell, d_sk, d_si, d_cs, d_ce, None)
    assert _call(*args) == 0, L.pbf_global_last_error()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert _call(*args) == 0, L.pbf_global_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_static_scratch_rejects_counts_beyond_capacity(pbf):
    L = pbf.load()
    cap = L.pbf_static_scratch_capacity()
    dummy = C.c_void_p(16)  # never dereferenced: the count is rejected first
    st = L.pbf_grid_build_static_scratch(
        dummy, cap + 1, _f3(pbf, (0, 0, 0)), _f3(pbf, (1, 1, 1)), 0.5, dummy, dummy, dummy,
        dummy, None)
    assert st == 4  # PBF_ERR_LENGTH
    assert "static scratch capacity" in L.pbf_global_last_error().decode()
