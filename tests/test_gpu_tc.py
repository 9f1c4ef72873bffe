"""tcgen05 TF32 GEMM (tensor cores, TMEM accumulator) through the C-ABI.

Integer-valued operands are exact in TF32 and their products sum exactly in FP32, so
the tensor-core result must match bit for bit: this pins the TMA swizzle, the UMMA
descriptors and the TMEM read-out.  Random operands check the TF32 error bound.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc(lib, A, B):
    bt, M, K = A.shape
    N = B.shape[1]
    D = np.zeros((bt, M, N), np.float32)
    A = np.ascontiguousarray(A, np.float32)
    B = np.ascontiguousarray(B, np.float32)
    rc = lib.forge_gpu_selftest_tc_gemm(M, N, K, bt, A.ctypes.data_as(C.c_void_p), B.ctypes.data_as(C.c_void_p),
                                        D.ctypes.data_as(C.c_void_p))
    assert rc == 0, lib.forge_gpu_last_error()
    return D


@pytest.mark.parametrize("M,N,K,bt", [(128, 128, 32, 1), (256, 384, 96, 1), (200, 130, 70, 2), (129, 257, 1000, 1),
                                      (1024, 512, 640, 3)])
def test_tc_gemm_exact_on_integers(lib, M, N, K, bt):
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-8, 9, size=(bt, M, K)).astype(np.float32)
    B = rng.integers(-8, 9, size=(bt, N, K)).astype(np.float32)
    D = _tc(lib, A, B)
    ref = np.einsum("bmk,bnk->bmn", A.astype(np.float64), B.astype(np.float64))
    assert np.array_equal(D.astype(np.float64), ref)


def test_tc_gemm_tf32_error_bound(lib):
    rng = np.random.default_rng(7)
    A = rng.standard_normal((1, 300, 512)).astype(np.float32)
    B = rng.standard_normal((1, 260, 512)).astype(np.float32)
    D = _tc(lib, A, B)
    ref = A[0].astype(np.float64) @ B[0].astype(np.float64).T
    # TF32 keeps 10 explicit mantissa bits: |err| <~ 2^-10 * sum |a||b|
    bound = 2.0 ** -9 * (np.abs(A[0]).astype(np.float64) @ np.abs(B[0]).astype(np.float64).T)
    assert np.all(np.abs(D[0] - ref) <= bound)


def _tf32(x):
    """Rounds toward zero to the 10-bit TF32 mantissa (the values are then exact in TF32)."""
    b = np.asarray(x, np.float32).view(np.uint32) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def test_tc_gemm_accumulation_bias_is_bounded(lib):
    """With TF32-exact all-positive operands the tensor core's FP32 accumulation truncates (measured
    -5.9e-5 relative at K = 8192 with one TMEM accumulator); the kernel accumulates each K block of 32
    alone and sums the blocks in round-to-nearest FP32 registers, which bounds the bias near -9e-8
    independently of K."""
    rng = np.random.default_rng(0)
    M = N = 256
    for K in (512, 8192):
        A = _tf32(rng.uniform(0.5, 1.0, (1, M, K)))
        B = _tf32(rng.uniform(0.5, 1.0, (1, N, K)))
        D = _tc(lib, A, B)
        ref = A[0].astype(np.float64) @ B[0].astype(np.float64).T
        rel = (D[0] - ref) / np.abs(ref).max()
        assert abs(float(rel.mean())) <= 3e-7, (K, float(rel.mean()))


def test_tc_gemm_bounded_wait_times_out_cleanly(lib):
    """Failure detection without a GPU fault: a GEMM whose second K block never arrives gives up its
    bounded mbarrier wait and returns FORGE_ERR_TIMEOUT (-5); the context then runs an exact GEMM."""
    rng = np.random.default_rng(5)
    A = rng.integers(-8, 9, size=(1, 256, 128)).astype(np.float32)
    B = rng.integers(-8, 9, size=(1, 192, 128)).astype(np.float32)
    D = np.zeros((1, 256, 192), np.float32)
    rc = lib.forge_gpu_selftest_tc_gemm_timeout(256, 192, 128, 1 << 14, A.ctypes.data_as(C.c_void_p),
                                                B.ctypes.data_as(C.c_void_p), D.ctypes.data_as(C.c_void_p))
    assert rc == -5, lib.forge_gpu_last_error()
    assert b"gave up" in lib.forge_gpu_last_error()
    D2 = _tc(lib, A, B)
    assert np.array_equal(D2[0].astype(np.float64), A[0].astype(np.float64) @ B[0].astype(np.float64).T)
