"""The tcgen05 BF16 GEMM primitive (TMEM accumulator, K-major shared-memory operands)
against a host GEMM on the same BF16 inputs: FP32 accumulation, tolerance
1e-5 relative to sum(|a*b|)."""
import ctypes as C

import numpy as np
import pytest

from realcausticsengine_gb300 import _native

pytestmark = pytest.mark.gpu


def to_bf16_bits(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)   # round to nearest even
    return r


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("K,N", [(16, 16), (64, 64), (80, 64), (64, 80), (128, 256), (96, 48)])
def test_tc_gemm_matches_host(K, N):
    lib = _native.lib()
    lib.rc_tc_gemm_selftest.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(K * 1000 + N)
    A = to_bf16_bits(rng.normal(size=(128, K)))
    B = to_bf16_bits(rng.normal(size=(N, K)))
    D = np.zeros((128, N), np.float32)
    rc = lib.rc_tc_gemm_selftest(K, N, A.ctypes.data, B.ctypes.data, D.ctypes.data)
    assert rc == 0
    a = bf16_bits_to_f32(A).astype(np.float64)
    b = bf16_bits_to_f32(B).astype(np.float64)
    want = a @ b.T
    scale = np.abs(a) @ np.abs(b).T
    assert np.all(np.abs(D - want) <= 1e-5 * scale + 1e-6), np.abs(D - want).max()


def test_bounded_wait_expires_and_context_survives():
    """A bounded mbarrier wait that nothing completes (no MMA in flight) must expire,
    free its TMEM and report RC_E_TIMEOUT; the next tensor-core launch must work."""
    lib = _native.lib()
    assert lib.rc_tc_wait_selftest(2048) == -6
    assert lib.rc_tc_wait_selftest(1) == -6
    rng = np.random.default_rng(5)
    A = to_bf16_bits(rng.normal(size=(128, 16)))
    B = to_bf16_bits(rng.normal(size=(16, 16)))
    D = np.zeros((128, 16), np.float32)
    assert lib.rc_tc_gemm_selftest(16, 16, A.ctypes.data, B.ctypes.data, D.ctypes.data) == 0
    want = bf16_bits_to_f32(A).astype(np.float64) @ bf16_bits_to_f32(B).astype(np.float64).T
    assert np.abs(D - want).max() < 1e-3
