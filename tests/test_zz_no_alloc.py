"""dsc_tc_gemm_noalloc: the tensor-core product on caller-owned device
memory with its scratch in a static device array.

On the GPU it must give the same Y as dsc_tc_gemm, bit for bit, on two
calls in a row with different shapes and split counts (the second call
reads nothing the first left in the scratch), leave the columns of Y past
Nc alone, and change the device's free memory by nothing.  Oversize shapes
are rejected before any device work, so that check also runs without a GPU.

This file is named to be collected last: it must pass both alone and after
every other test in the same process.
"""
import numpy as np
import pytest

from depsolver_gb300 import _native

SCRATCH = 32 << 20


def _case(rng, M, Nc, Kd):
    A32 = (rng.standard_normal((M, Kd)) * np.exp(rng.uniform(-3, 3, (M, 1)))).astype(np.float32)
    B = rng.standard_normal((Nc, Kd))
    return A32, B


def _existing(L, A32, B, splits):
    M, Kd = A32.shape
    Nc = B.shape[0]
    Y = np.zeros((M, Nc))
    _native.check(L.dsc_tc_gemm(M, Nc, Kd, np.ascontiguousarray(A32, dtype=np.float64),
                                np.ascontiguousarray(B), Y, splits, 1))
    return Y


@pytest.mark.gpu
def test_noalloc_matches_dsc_tc_gemm_on_two_calls_in_a_row(gpu):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch sees no CUDA device")
    L = gpu
    rng = np.random.default_rng(2024)
    # (M, Nc, Kd, splits): automatic split count on a ragged shape, then an
    # explicit one on another shape
    cases = [(1000, 128, 2500, 0), (300, 40, 1000, 3)]
    prepared = []
    for M, Nc, Kd, splits in cases:
        A32, B = _case(rng, M, Nc, Kd)
        lda = (Kd + 3) // 4 * 4 + 4   # padded rows: a stride that is not Kd
        ldb = Kd + 1
        ldy = Nc + 3
        dA = torch.zeros((M, lda), dtype=torch.float32, device="cuda")
        dA[:, :Kd] = torch.from_numpy(A32).cuda()
        dB = torch.zeros((Nc, ldb), dtype=torch.float64, device="cuda")
        dB[:, :Kd] = torch.from_numpy(B).cuda()
        dY = torch.full((M, ldy), float("nan"), dtype=torch.float64, device="cuda")
        prepared.append((M, Nc, Kd, splits, A32, B, lda, ldb, ldy, dA, dB, dY))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream

    free = []
    for M, Nc, Kd, splits, A32, B, lda, ldb, ldy, dA, dB, dY in prepared:
        f0 = torch.cuda.mem_get_info()[0]
        _native.check(L.dsc_tc_gemm_noalloc(M, Nc, Kd, dA.data_ptr(), lda, dB.data_ptr(), ldb,
                                            dY.data_ptr(), ldy, splits, stream))
        free.append((f0, torch.cuda.mem_get_info()[0]))
    # the second call (module and scratch already loaded) allocates nothing
    assert free[1][0] == free[1][1], free

    for M, Nc, Kd, splits, A32, B, lda, ldb, ldy, dA, dB, dY in prepared:
        Y = dY.cpu().numpy()
        ref = _existing(L, A32, B, splits)
        assert np.array_equal(Y[:, :Nc], ref), float(np.nanmax(np.abs(Y[:, :Nc] - ref)))
        assert np.isnan(Y[:, Nc:]).all()
        # and both are the FP32-accurate product
        exact = A32.astype(np.float64) @ B.T
        bound = np.abs(A32.astype(np.float64)) @ np.abs(B).T
        assert np.all(np.abs(ref - exact) <= 2e-6 * bound)


@pytest.mark.gpu
def test_noalloc_rejects_host_pointers(gpu):
    A = np.zeros((128, 32), dtype=np.float32)
    B = np.zeros((16, 32))
    Y = np.zeros((128, 16))
    st = gpu.dsc_tc_gemm_noalloc(128, 16, 32, A.ctypes.data, 32, B.ctypes.data, 32, Y.ctypes.data,
                                 16, 1, None)
    assert st == 2
    assert b"device memory" in gpu.dsc_last_error()


def test_noalloc_rejects_oversize_before_device_work(native):
    """Shapes whose scratch exceeds the static array fail with DSC_ERR_ARG
    and a message giving both sizes, with or without a GPU."""
    M, Nc, Kd = 60000, 160, 4       # one partial tile alone: 60000 * 160 * 4 B > 32 MiB
    A = np.zeros((M, Kd), dtype=np.float32)
    B = np.zeros((Nc, Kd))
    Y = np.zeros((M, Nc))
    for splits in (0, 1):
        st = native.dsc_tc_gemm_noalloc(M, Nc, Kd, A.ctypes.data, Kd, B.ctypes.data, Kd,
                                        Y.ctypes.data, Nc, splits, None)
        assert st == 2
        msg = native.dsc_last_error().decode()
        assert "scratch" in msg and str(SCRATCH) in msg, msg
    # an explicit split count that does not fit is not lowered silently
    M, Nc, Kd = 4096, 128, 4096
    A = np.zeros((M, Kd), dtype=np.float32)
    B = np.zeros((Nc, Kd))
    Y = np.zeros((M, Nc))
    st = native.dsc_tc_gemm_noalloc(M, Nc, Kd, A.ctypes.data, Kd, B.ctypes.data, Kd, Y.ctypes.data,
                                    Nc, 64, None)
    assert st == 2 and b"64 splits" in native.dsc_last_error()
