"""The split-BF16 tcgen05 GEMM (the engine's tensor-core Legendre contraction) against a float64 product.

Expected accuracy (relative Frobenius error of D = A B^T, FP32 accumulation): one BF16 product ~3e-3, the
three-term hi/lo split ~1e-5 (about 16 significant bits), the six-term hi/mid/lo split at the FP32 level."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_gemm(engine, A, B, terms, layout=0):
    lib = engine.load_library()
    f = lib.lmw_tc_gemm_selftest
    FP = ctypes.POINTER(ctypes.c_float)
    f.argtypes = [FP, FP, FP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    f.restype = ctypes.c_int
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    N, K = B.shape
    D = np.zeros((128, N), np.float32)
    st = ctypes.c_int(-1)
    engine._check(f(A.ctypes.data_as(FP), B.ctypes.data_as(FP), D.ctypes.data_as(FP), N, K, terms, layout, ctypes.byref(st)))
    assert st.value == 0, "a wait on the tensor cores ran out"
    return D


def rel(D, A, B):
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    return np.linalg.norm(D - ref) / np.linalg.norm(ref)


@pytest.mark.parametrize("N,K", [(16, 16), (64, 128), (48, 80), (256, 192), (128, 320)])
def test_split_gemm_accuracy(engine, N, K):
    rng = np.random.default_rng(N * 1000 + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    e1 = rel(run_gemm(engine, A, B, 1), A, B)
    e3 = rel(run_gemm(engine, A, B, 3), A, B)
    e6 = rel(run_gemm(engine, A, B, 6), A, B)
    print(f"N={N} K={K}: 1 term {e1:.2e}, 3 terms {e3:.2e}, 6 terms {e6:.2e}")
    assert e1 < 1e-2
    assert e3 < 5e-5
    assert e6 < 5e-6  # the tensor-core FP32 accumulation grows with K: 5e-8 at K = 16, 2e-6 at K = 320
    assert e6 < e3 < e1
