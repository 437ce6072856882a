"""The mixed path's tcgen05 pipelines in isolation: one 128 x N tile
C = A B^T through occ_xc_selftest_tf32_gemm, against a float64 product.

exact = 0  3xTF32 (hi*hi + hi*lo + lo*hi), used for the V_xc contraction
exact = 1  exact-grid split (two 8-bit integer-grid slices and a TF32 tail
           per value, relative to a power-of-two row bound), used for the
           density contraction
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(exact, A, B):
    from occ_gb300.xc import _context
    ctx = _context(0)
    lib = ctx.lib
    lib.occ_xc_selftest_tf32_gemm.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                              C.c_void_p, C.c_void_p]
    N, K = B.shape
    Cm = np.zeros((128, N), dtype=np.float32)
    rc = lib.occ_xc_selftest_tf32_gemm(ctx.h, exact, N, K, A.ctypes.data, B.ctypes.data,
                                       Cm.ctypes.data)
    assert rc == 0, ctx.error()
    return Cm


@pytest.mark.parametrize("N,K", [(32, 32), (64, 64), (128, 128), (256, 32), (256, 512), (96, 160)])
def test_tf32x3_tile(N, K):
    rng = np.random.default_rng(N * 1000 + K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    Cm = _gemm(0, A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    # 3xTF32 keeps about FP32 accuracy; a plain TF32 product would be ~1e-3
    assert np.max(np.abs(Cm - ref) / scale) < 2e-6


@pytest.mark.parametrize("N,K", [(32, 32), (128, 128), (64, 512), (96, 160)])
def test_exact_split_tile(N, K):
    rng = np.random.default_rng(N * 7 + K)
    # rows of very different magnitudes, as AO values and density columns have
    A = (rng.standard_normal((128, K)) * 10.0 ** rng.uniform(-6, 2, (128, 1))).astype(np.float32)
    B = (rng.standard_normal((N, K)) * 10.0 ** rng.uniform(-4, 1, (N, 1))).astype(np.float32)
    Cm = _gemm(1, A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    err = np.max(np.abs(Cm - ref) / scale)
    print(f"exact split {N}x{K}: max error / (|A||B|) = {err:.2e}")
    assert err < 1e-6


def test_accumulation_bias():
    """All-positive operands.  The TMEM accumulator truncates, so 3xTF32 shows a
    one-sided error that grows with K; the exact-grid split has none beyond the
    final FP32 rounding."""
    N, K = 128, 512
    rng = np.random.default_rng(7)
    A = rng.uniform(0.5, 1.5, (128, K)).astype(np.float32)
    B = rng.uniform(0.5, 1.5, (N, K)).astype(np.float32)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    bias3 = float(((_gemm(0, A, B) - ref) / ref).mean())
    biasx = float(((_gemm(1, A, B) - ref) / ref).mean())
    print(f"mean relative error: 3xTF32 {bias3:.3e}, exact split {biasx:.3e}")
    assert bias3 < -1e-7          # the truncation this design works around
    assert abs(biasx) < 2e-8      # unbiased to FP32 rounding
