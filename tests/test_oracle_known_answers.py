"""Pins the CPU oracle against the reference's own known-answer tests.

Every case in cases.py restates one test of the reference
(test/test_spatial_grid.cu, test/test_neighbors.cu, test/test_pbf_solver_kernels.cu,
test/test_correctness.cu, test/test_collision_*.cu, test/test_pbf_solver.cu);
the same cases run on the GPU against the CUDA library in
test_gpu_known_answers.py.
"""

import pytest

from backends import OracleBackend
from cases import ALL_CASES


@pytest.fixture(scope="module", params=[32, 64], ids=["fp32", "fp64"])
def backend(request):
    return OracleBackend(request.param)


STAGE_ONLY_FP32 = {"case_grid", "case_neighbors", "case_lambda", "case_delta", "case_scorr",
                   "case_correctness", "case_xsph", "case_vorticity", "case_container",
                   "case_sphere", "case_box", "case_plane", "case_resolve", "case_collision"}


@pytest.mark.parametrize("case", ALL_CASES, ids=[c.__name__ for c in ALL_CASES])
def test_oracle_case(case, backend):
    # The stage functions of the oracle exist in FP32 mirror form only; the
    # whole-solver cases run in both precisions.
    if backend.precision == 64 and any(case.__name__.startswith(p) for p in STAGE_ONLY_FP32):
        pytest.skip("stage functions are FP32 only")
    case(backend)
