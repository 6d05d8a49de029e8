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


@pytest.mark.parametrize("h", [0.016, 0.05, 0.036, 0.1, 1.0, 0.002, 3.0])
def test_colour_field_gradient_in_fp32_matches_double(h):
    """The colour field's spiky gradient float(k x x) (double in the
    reference) is formed in FP32 with a double fallback near rounding
    midpoints; every float x in (0, 1] must give the double result."""
    import torch
    from fluidsurfacereconstructiongpu_gb300 import _native as N
    torch.cuda.init()
    h2 = float(np.float32(np.float32(h) * np.float32(h)))
    k = -45.0 / (3.1415926535 * h2 * h2)   # as launch_colorfield forms it
    checked, bad = ctypes.c_uint64(), ctypes.c_uint64()
    N.check(N.lib.fsr_check_spiky_grad(k, ctypes.byref(checked), ctypes.byref(bad)))
    assert checked.value == 0x3F800000
    assert bad.value == 0, (h, bad.value)
