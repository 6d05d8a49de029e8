"""The smoothing and covariance kernels divide distances by the neighbour
radius R with an FMA refinement of d x RN(1/R) (Markstein's theorem) instead
of the IEEE division; every float d in [0, 1.01 R] must give __fdiv_rn's
result, for the radii the tests and the benchmark use and a few others."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R", [0.016, 0.032, 0.1, 0.07, 0.0125, 1.0, 3.7, 1e-3, 123.456, 7e-6])
def test_exact_division_matches_ieee(R):
    import torch
    from fluidsurfacereconstructiongpu_gb300 import _native as N
    torch.cuda.init()
    checked, bad = ctypes.c_uint64(), ctypes.c_uint64()
    N.check(N.lib.fsr_check_division(float(np.float32(R)), ctypes.byref(checked), ctypes.byref(bad)))
    assert checked.value > 10**8
    assert bad.value == 0, (R, bad.value)
