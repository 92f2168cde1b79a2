"""The tcgen05 split-K GEMM (3xTF32, and 3xFP16 on scaled fp16 pairs)
against an FP64 product (NumPy).

Bar: |Y - A B^T| <= 2e-6 * (|A| |B|^T) elementwise -- the FP32-level
accuracy the mixed inner solver relies on -- for ragged shapes (rows not a
multiple of 128, k not a multiple of 32 / 64, columns not a multiple of 16).
"""
import numpy as np
import pytest

from depsolver_gb300 import _native

pytestmark = pytest.mark.gpu


def _run(L, A, B, splits, a_in_smem=1):
    M, Kd = A.shape
    Nc = B.shape[0]
    Y = np.zeros((M, Nc))
    _native.check(L.dsc_tc_gemm(M, Nc, Kd, np.ascontiguousarray(A), np.ascontiguousarray(B), Y,
                                splits, a_in_smem))
    return Y


@pytest.mark.parametrize("a_in_smem", [0, 1, 2, 3])
@pytest.mark.parametrize("M,Nc,Kd,splits", [
    (128, 16, 32, 1),      # one tile, one k-block
    (300, 40, 1000, 1),    # ragged everything, one split
    (300, 128, 1000, 4),   # split-K
    (1000, 128, 2500, 0),  # automatic split count
    (257, 100, 77, 3),
])
def test_tc_gemm_matches_fp64(gpu, M, Nc, Kd, splits, a_in_smem):
    rng = np.random.default_rng(M + Nc + Kd)
    A = rng.standard_normal((M, Kd)) * np.exp(rng.uniform(-3, 3, (M, 1)))
    B = rng.standard_normal((Nc, Kd))
    Y = _run(gpu, A, B, splits, a_in_smem)
    ref = A @ B.T
    bound = np.abs(A) @ np.abs(B).T
    assert np.all(np.abs(Y - ref) <= 2e-6 * bound + 1e-300), float(np.max(np.abs(Y - ref) / bound))


def test_tc_gemm_beats_plain_tf32(gpu):
    """Three products are needed: one TF32 product alone would miss by ~1e-3."""
    rng = np.random.default_rng(7)
    A = rng.standard_normal((256, 512))
    B = rng.standard_normal((32, 512))
    Y = _run(gpu, A, B, 2)
    rel = np.abs(Y - A @ B.T).max() / np.abs(A @ B.T).max()
    assert rel < 1e-5


def test_tc_gemm_f16_scales_rows_and_columns(gpu):
    """3xFP16: rows of A and of B spread over 2^-40 .. 2^40 (far outside
    fp16's range; the products stay inside FP32's, where the partial tiles
    live) keep the FP32-level bound: each row's power-of-two scale is
    multiplied back out exactly."""
    rng = np.random.default_rng(11)
    M, Nc, Kd = 400, 96, 700
    A = rng.standard_normal((M, Kd)) * np.exp2(rng.integers(-40, 40, (M, 1)))
    A[:, ::7] *= 1e-9   # small entries next to large ones in the same row
    B = rng.standard_normal((Nc, Kd)) * np.exp2(rng.integers(-40, 40, (Nc, 1)))
    B[3] = 0.0           # an all-zero operand row
    Y = _run(gpu, A, B, 0, 3)
    ref = A @ B.T
    bound = np.abs(A) @ np.abs(B).T
    assert np.all(np.abs(Y - ref) <= 2e-6 * bound + 1e-300), float(np.nanmax(np.abs(Y - ref) / bound))
    assert np.all(Y[:, 3] == 0.0)


@pytest.mark.parametrize("M,Nc,Kd", [
    (300, 384, 10000),  # three splits of at most 4096, two MMAs of 192 columns
    (257, 256, 4096),   # one full split
    (128, 16, 77),      # ragged k
    (1000, 200, 9000),
])
def test_tc_gemm_digits_exact(gpu, M, Nc, Kd):
    """The digit product (mode 4) is exact: integer operands |A| <= 32,
    |B| <= 128 give integer partial sums of at most 2^24 per split, which
    the FP32 accumulator must hold without rounding whatever its order."""
    rng = np.random.default_rng(M * Nc + Kd)
    A = rng.integers(-32, 33, (M, Kd))
    B = rng.integers(-128, 129, (Nc, Kd))
    # rows at the bound: every product +4096 (the partial sums reach 2^24)
    A[0] = 32
    B[0] = 128
    A[1] = -32
    B[1] = np.where(np.arange(Kd) % 2 == 0, 128, -127)  # alternating, no cancellation to zero
    Y = _run(gpu, A.astype(float), B.astype(float), 0, 4)
    ref = A.astype(np.int64) @ B.astype(np.int64).T
    assert np.array_equal(Y, ref.astype(float)), float(np.abs(Y - ref).max())
