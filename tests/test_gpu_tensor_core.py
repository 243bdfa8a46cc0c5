"""tcgen05 BF16 MMA through the library's self-test GEMM, against numpy.

The learned-correction kernels stage activations once in shared memory and
read them both as a K-major A operand (forward) and as an MN-major B operand
(weight gradients); this pins both layouts.  Tolerance: FP32 accumulation of
exact BF16 products, |C - C_ref| <= 1e-5 * (|A| |B|^T) elementwise.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_bf16_bits(x):
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)   # round to nearest even
    return r


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("n,k,a_mn,b_mn", [(64, 64, 0, 0), (16, 64, 0, 0), (64, 32, 0, 0),
                                           (64, 128, 0, 1), (128, 128, 1, 1), (64, 32, 1, 0),
                                           (128, 64, 0, 0)])
def test_tc_gemm(lib, n, k, a_mn, b_mn):
    rng = np.random.default_rng(n * 1000 + k + 7 * a_mn + 13 * b_mn)
    A = to_bf16_bits(rng.standard_normal((128, k)))
    B = to_bf16_bits(rng.standard_normal((n, k)))
    C = np.zeros((128, n), dtype=np.float32)
    f = lib.gsgpu_tc_gemm_selftest
    f.restype = ctypes.c_int
    rc = f(n, k, a_mn, b_mn, A.ctypes.data_as(ctypes.c_void_p), B.ctypes.data_as(ctypes.c_void_p),
           C.ctypes.data_as(ctypes.c_void_p))
    assert rc == 0
    Af, Bf = from_bf16_bits(A).astype(np.float64), from_bf16_bits(B).astype(np.float64)
    ref = Af @ Bf.T
    bound = 1e-5 * (np.abs(Af) @ np.abs(Bf).T) + 1e-30
    assert np.all(np.abs(C - ref) <= bound), float(np.max(np.abs(C - ref) / bound))
