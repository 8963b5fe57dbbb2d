"""Tensor-core path of the learned relocation proposal (GPU only)."""
import ctypes as C

import numpy as np
import pytest

from msplat_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    """float32 values exactly representable in bfloat16 -> their 16-bit patterns."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32)
    assert np.all((b & 0xFFFF) == 0)
    return (b >> 16).astype(np.uint16)


@pytest.mark.parametrize("n,k", [(16, 16), (32, 32), (64, 64), (16, 64), (64, 16)])
def test_tc_gemm_probe(n, k):
    L = N.lib()
    L.msplat_tc_gemm_check.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    rng = np.random.default_rng(n * 100 + k)
    A = rng.integers(-4, 5, (128, k)).astype(np.float32)
    B = rng.integers(-4, 5, (n, k)).astype(np.float32) * 0.5
    D = np.zeros((128, n), np.float32)
    a, b = _bf16_bits(A), _bf16_bits(B)
    rc = L.msplat_tc_gemm_check(a.ctypes.data, b.ctypes.data, D.ctypes.data, n, k)
    assert rc == 0
    np.testing.assert_array_equal(D, A @ B.T)      # small integers: exact in F32
