"""The split hi/lo BF16 tensor-core product (tcgen05.mma with FP32 accumulation in tensor
memory), the primitive of the shared-grid line-of-sight projection, against numpy in FP64.

Inputs that BF16 represents exactly (small integers times powers of two) must come out
to FP32 accumulation accuracy; random FP32 inputs over partial 128 x 128 tiles and several
64-deep K tiles within 1e-4 of sum_k |A||B| per element (the split keeps ~16 significant
bits of each operand; the A_lo B_lo term and FP32 accumulation are the remaining error)."""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib

pytestmark = pytest.mark.gpu


def gemm(A, B):
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M, K = A.shape
    N = B.shape[0]
    D = np.full((M, N), np.nan, dtype=np.float32)
    fp = C.POINTER(C.c_float)
    rc = _lib.load().cambgpu_gemm_bf16x3(A.ctypes.data_as(fp), B.ctypes.data_as(fp), M, N, K, D.ctypes.data_as(fp))
    assert rc == 0, _lib.load().cambgpu_last_error()
    return D


def test_exact_operands_one_tile():
    rng = np.random.default_rng(1)
    A = rng.integers(-8, 9, size=(128, 64)).astype(np.float32) / 4
    B = rng.integers(-8, 9, size=(128, 64)).astype(np.float32) / 8
    D = gemm(A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    np.testing.assert_allclose(D, ref, rtol=0, atol=1e-4)


@pytest.mark.parametrize("shape", [(200, 300, 500), (97, 1024, 1000), (128, 256, 2000)])
def test_random_operands_partial_tiles(shape):
    M, N, K = shape
    rng = np.random.default_rng(M + N + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = (rng.normal(size=(N, K)) * np.exp(rng.normal(size=(N, 1)))).astype(np.float32)
    D = gemm(A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    bound = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert np.all(np.isfinite(D))
    assert np.max(np.abs(D - ref) / bound) < 1e-4
