"""The reference's own kernels compiled by nvcc (the "reference GPU" timing
line of the bench) against their CPU build: the driver reproduces the
reference's loop.  Not bitwise: nvcc contracts a*b+c into fma and CUDA's pow
is not glibc's; 1e-9 m."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import bumpy_case

pytestmark = pytest.mark.gpu


def test_reference_gpu_build_matches_its_cpu_build():
    if O.ref_gpu_lib() is None or O.ref_lib() is None:
        pytest.skip("reference builds unavailable")
    case = bumpy_case(R=48, C=40, seed=3, t_end=30.0, dt=0.05)
    cpu = O.run_reference(case, nthreads=4)
    gpu = O.run_reference(case, gpu=True)
    assert gpu["iters"] == cpu["iters"] == 300
    for k in ("h", "um", "vn", "uu", "vv"):
        assert np.abs(gpu[k] - cpu[k]).max() <= 1e-9, k
