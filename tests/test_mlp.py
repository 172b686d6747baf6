"""Solid-angle surrogate network: the tensor-core (tcgen05) kernels against
the NumPy restatement in oracle/mlp_reference.py."""
import ctypes as C

import numpy as np
import pytest


def ref():
    from oracle import mlp_reference
    return mlp_reference


def test_reference_layout_matches_engine_parameter_count():
    from xmimsim_gb300 import abi
    lib = abi.load()
    lib.xmi_mlp_nparam.restype = C.c_int
    assert lib.xmi_mlp_nparam() == ref().NPARAM


def test_bf16_rounding_is_nearest_even():
    r = ref()
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], dtype=np.float32)
    y = r.bf16(x)
    assert y[0] == 1.0 and y[1] == 1.0 and y[2] == np.float32(1.0078125)
    assert abs(y[3] - x[3]) <= abs(x[3]) * 2 ** -8


@pytest.mark.gpu
def test_forward_kernel_matches_reference():
    from xmimsim_gb300 import abi
    r = ref()
    lib = abi.load()
    fp = C.POINTER(C.c_float)
    lib.xmi_gpu_mlp_forward.restype = C.c_int
    lib.xmi_gpu_mlp_forward.argtypes = [fp, C.c_int, fp, fp]
    theta = r.init_params(3)
    rng = np.random.default_rng(4)
    n = 1000  # not a multiple of the 128-row tile
    x = rng.uniform(-1.0, 1.0, size=(n, 3)).astype(np.float32)
    out = np.zeros(n, dtype=np.float32)
    assert lib.xmi_gpu_mlp_forward(theta.ctypes.data_as(fp), n, x.ctypes.data_as(fp), out.ctypes.data_as(fp)) == 1, \
        abi.last_error()
    y = r.forward(theta, x)
    err = np.abs(out - y)
    assert np.median(err) < 2e-3 * (1 + np.median(np.abs(y)))
    assert err.max() < 2e-2 * (1 + np.abs(y).max())
