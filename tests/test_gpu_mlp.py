"""Tensor-core (tcgen05) building blocks of the MLP surrogate against numpy:
BF16-rounded operands, FP32 accumulation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16(x):
    """round-to-nearest-even to BF16, kept in float32"""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


@pytest.mark.parametrize("n,k", [(16, 16), (64, 16), (64, 64), (128, 32), (16, 64)])
def test_tc_gemm_matches_numpy(swe, n, k):
    rng = np.random.default_rng(n * 100 + k)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    d = swe.tc_gemm_check(a, b)
    ref = bf16(a).astype(np.float64) @ bf16(b).astype(np.float64).T
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-4), np.abs(d - ref).max()
