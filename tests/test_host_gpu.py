"""GPU tests of the host-buffer entry points (tsqr_s_host / tsqr_d_host):
A in host memory, Q and R returned to host memory, the copies pipelined with
the level-0 kernels in chunks of tiles.

Bar: the same results as the device entry point on the same matrix (the
tree and the kernels are the same; level 0 is only launched chunk by chunk),
within 1e-6 of max|R| for R and 1e-6 for Q, and the plain-path parity bar
against the FP64 oracle (backward error and orthogonality <= 10 n u).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_colmajor(A, pinned=True, ld=None):
    import torch
    m, n = A.shape
    ld = ld or m
    buf = torch.zeros((n, ld), dtype=torch.float32 if A.dtype == np.float32 else torch.float64,
                      pin_memory=pinned)
    buf[:, :m].copy_(torch.from_numpy(np.ascontiguousarray(A.T)))
    return buf.t()[:m]


def to_np(x):
    return x.t().contiguous().numpy().T


def device_result(tg, A, precision):
    import torch
    m, n = A.shape
    d = tg.empty_colmajor(m, n, torch.float32 if A.dtype == np.float32 else torch.float64, "cuda")
    d.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    R = tg.tsqr_(d, precision=precision)
    torch.cuda.synchronize()
    return d.t().contiguous().cpu().numpy().T, R.t().contiguous().cpu().numpy().T


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("m,n", [(1, 1), (513, 32), (27648, 32), (70001, 17), (262144, 8), (4096, 16)])
def test_host_entry_matches_device_entry(orc, cuda, tg, dtype, m, n):
    import torch
    A = orc.fill_uniform(m, n, dtype, seed=31)
    hA = host_colmajor(A)
    Q, R = tg.tsqr_host_(hA)
    torch.cuda.synchronize()
    Q, R = to_np(Q), to_np(R)
    Qd, Rd = device_result(tg, A, "plain")
    assert np.abs(R - Rd).max() <= 1e-6 * np.abs(Rd).max()
    assert np.abs(Q - Qd).max() <= 1e-6
    u = 2.0 ** -24 if dtype == np.float32 else 2.0 ** -53
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, met


@pytest.mark.parametrize("m,n", [(300000, 64), (1000000, 32), (5000, 13)])
def test_host_entry_precision_form(orc, cuda, tg, m, n):
    import torch
    A = orc.fill_uniform(m, n, np.float32, seed=32)
    Q, R = tg.tsqr_host_(host_colmajor(A), precision="tf32x3")
    torch.cuda.synchronize()
    Q, R = to_np(Q), to_np(R)
    Qd, Rd = device_result(tg, A, "tf32x3")
    assert np.abs(R - Rd).max() <= 1e-6 * np.abs(Rd).max()
    assert np.abs(Q - Qd).max() <= 1e-6
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met


def test_host_entry_padded_and_pageable(orc, cuda, tg):
    """Leading dimensions above m on the host side, and pageable (unpinned)
    buffers, whose copies cannot overlap but must still be correct."""
    import torch
    m, n = 20000, 24
    A = orc.fill_uniform(m, n, np.float32, seed=33)
    hA = host_colmajor(A, pinned=False, ld=m + 7)
    Q = torch.zeros((n, m + 3), dtype=torch.float32).t()[:m]
    R = torch.zeros((n, n + 1), dtype=torch.float32).t()[:n]
    tg.tsqr_host_(hA, Q, R)
    torch.cuda.synchronize()
    Qd, Rd = device_result(tg, A, "plain")
    assert np.abs(to_np(R) - Rd).max() <= 1e-6 * np.abs(Rd).max()
    assert np.abs(to_np(Q) - Qd).max() <= 1e-6
    assert np.array_equal(to_np(hA), A)  # A is only read


def test_host_entry_rejects_bad_arguments(cuda, tg):
    import ctypes
    import torch
    L = tg.lib()
    o = tg._opts("plain")
    a = torch.zeros((4, 100), dtype=torch.float32, pin_memory=True)
    q = torch.zeros((4, 100), dtype=torch.float32, pin_memory=True)
    r = torch.zeros((4, 4), dtype=torch.float32, pin_memory=True)
    w = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    args = lambda m, n, lda, ldq, ldr: (m, n, a.data_ptr(), lda, q.data_ptr(), ldq, r.data_ptr(), ldr,
                                        w.data_ptr(), 1 << 20, ctypes.byref(o), None)
    assert L.tsqr_s_host(*args(100, 4, 99, 100, 4)) == 1   # lda < m
    assert L.tsqr_s_host(*args(100, 4, 100, 99, 4)) == 1   # ldq < m
    assert L.tsqr_s_host(*args(100, 4, 100, 100, 3)) == 1  # ldr < n
    assert L.tsqr_s_host(*args(3, 4, 100, 100, 4)) == 1    # m < n
    assert L.tsqr_s_host(100, 4, a.data_ptr(), 100, q.data_ptr(), 100, r.data_ptr(), 4, w.data_ptr(), 16,
                         ctypes.byref(o), None) == 3      # workspace too small
