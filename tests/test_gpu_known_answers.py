"""The reference's known-answer tests, run through the C ABI on the GPU.

Same cases as test_oracle_known_answers.py (cases.py), backend = libpbf103.
"""

import pytest

from backends import CudaBackend
from cases import ALL_CASES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    return CudaBackend()


@pytest.mark.parametrize("case", ALL_CASES, ids=[c.__name__ for c in ALL_CASES])
def test_cuda_case(case, backend):
    case(backend)
