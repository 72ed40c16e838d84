"""GPU tests of the implicit-Q form (tsqr_*_factor, tsqr_*_apply_qt,
tsqr_*_form_q), which the reference does not have (it always forms the
explicit Q, kernelQR.h:224-290).

Bars:
  * factor then form_q gives bit-for-bit the Q and R of tsqr_ (the same
    kernels on the same tree, only split into two calls);
  * apply_qt(C) equals Q^T C formed with the explicit Q in FP64, within
    20 n u ||C||_F (u = 2^-24 / 2^-53);
  * a least-squares solve x = R^-1 Q^T b matches the FP64 LAPACK solution
    within 1e-4 (FP32) / 1e-10 (FP64) relative;
  * C is only read.
Shapes cover the ragged last tile, a single-tile (root-only) tree, the
1024-row tiles of n <= 8, several 32-column blocks of C and k = 1.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(tg, X):
    import torch
    m, n = X.shape
    dt = torch.float32 if X.dtype == np.float32 else torch.float64
    d = tg.empty_colmajor(m, n, dt, "cuda")
    d.copy_(torch.from_numpy(np.ascontiguousarray(X)))
    return d


def to_host(x):
    return x.t().contiguous().cpu().numpy().T


@pytest.mark.parametrize("m,n,dtype", [(27648, 32, np.float32), (70001, 17, np.float32), (100, 64, np.float32),
                                       (5000, 8, np.float32), (262144, 64, np.float32), (1000, 13, np.float64),
                                       (27648, 32, np.float64)])
def test_factor_then_form_q_equals_tsqr(orc, cuda, tg, m, n, dtype):
    import torch
    A0 = orc.fill_uniform(m, n, dtype, seed=51)
    Q1 = to_dev(tg, A0)
    R1 = tg.tsqr_(Q1)
    A2 = to_dev(tg, A0)
    fac = tg.factor_(A2)
    tg.form_q_(fac)
    torch.cuda.synchronize()
    assert torch.equal(Q1, A2)
    assert torch.equal(R1, fac.R)


@pytest.mark.parametrize("m,n,k,dtype", [(27648, 32, 1, np.float32), (27648, 32, 70, np.float32),
                                         (70001, 17, 33, np.float32), (100, 64, 5, np.float32),
                                         (5000, 8, 32, np.float32), (262144, 64, 7, np.float32),
                                         (1000, 13, 3, np.float64), (27648, 32, 40, np.float64)])
def test_apply_qt_matches_explicit_q(orc, cuda, tg, m, n, k, dtype):
    import torch
    A0 = orc.fill_uniform(m, n, dtype, seed=52)
    C0 = orc.fill_uniform(m, k, dtype, seed=53)
    Q = to_dev(tg, A0)
    tg.tsqr_(Q)
    fac = tg.factor_(to_dev(tg, A0))
    C = to_dev(tg, C0)
    D = tg.apply_qt_(fac, C)
    torch.cuda.synchronize()
    ref = to_host(Q).astype(np.float64).T @ C0.astype(np.float64)
    u = 2.0 ** -24 if dtype == np.float32 else 2.0 ** -53
    err = np.linalg.norm(to_host(D).astype(np.float64) - ref)
    assert err <= 20 * n * u * np.linalg.norm(C0.astype(np.float64)), err
    assert np.array_equal(to_host(C), C0)  # C is only read


@pytest.mark.parametrize("m,n,dtype,tol", [(100000, 32, np.float32, 1e-4), (20000, 24, np.float64, 1e-10)])
def test_least_squares_solve(orc, cuda, tg, m, n, dtype, tol):
    import torch
    rng = np.random.default_rng(54)
    A0 = rng.standard_normal((m, n)).astype(dtype)
    x_true = rng.standard_normal(n)
    b0 = (A0.astype(np.float64) @ x_true + 0.01 * rng.standard_normal(m)).astype(dtype)[:, None]
    fac = tg.factor_(to_dev(tg, A0))
    qtb = tg.apply_qt_(fac, to_dev(tg, b0))
    torch.cuda.synchronize()
    R = to_host(fac.R).astype(np.float64)
    x = np.linalg.solve(np.triu(R), to_host(qtb).astype(np.float64)[:, 0])
    x_ref = np.linalg.lstsq(A0.astype(np.float64), b0.astype(np.float64)[:, 0], rcond=None)[0]
    assert np.linalg.norm(x - x_ref) <= tol * np.linalg.norm(x_ref)


def test_implicit_rejects_bad_arguments(cuda, tg):
    import ctypes
    import torch
    L = tg.lib()
    a = tg.empty_colmajor(100, 8, torch.float32, "cuda")
    r = tg.empty_colmajor(8, 8, torch.float32, "cuda")
    w = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    o = tg._opts("tf32x3")
    assert L.tsqr_s_factor(100, 8, a.data_ptr(), 100, r.data_ptr(), 8, w.data_ptr(), 1 << 20, ctypes.byref(o),
                           None) == 2  # plain precision only
    c = tg.empty_colmajor(100, 3, torch.float32, "cuda")
    d = tg.empty_colmajor(8, 3, torch.float32, "cuda")
    args = lambda m, n, ldv, ldc, ldd, cwb: (m, n, a.data_ptr(), ldv, w.data_ptr(), 1 << 20, 3, c.data_ptr(), ldc,
                                             d.data_ptr(), ldd, w.data_ptr(), cwb, None)
    assert L.tsqr_s_apply_qt(*args(100, 8, 99, 100, 8, 1 << 20)) == 1   # ldv < m
    assert L.tsqr_s_apply_qt(*args(100, 8, 100, 99, 8, 1 << 20)) == 1   # ldc < m
    assert L.tsqr_s_apply_qt(*args(100, 8, 100, 100, 7, 1 << 20)) == 1  # ldd < n
    assert L.tsqr_s_apply_qt(*args(100, 80, 100, 100, 80, 1 << 20)) == 2  # n > 64
    assert L.tsqr_s_form_q(100, 8, a.data_ptr(), 99, w.data_ptr(), 1 << 20, None) == 1


def test_implicit_with_padded_leading_dimensions(orc, cuda, tg):
    """lda > m for the factored A, ldc > m for C and ldd > n for D."""
    import torch
    m, n, k = 30001, 24, 6
    A0 = orc.fill_uniform(m, n, np.float32, seed=55)
    C0 = orc.fill_uniform(m, k, np.float32, seed=56)
    A = tg.empty_colmajor(m, n, torch.float32, "cuda", ld=m + 5)
    A.copy_(torch.from_numpy(np.ascontiguousarray(A0)))
    C = tg.empty_colmajor(m, k, torch.float32, "cuda", ld=m + 3)
    C.copy_(torch.from_numpy(np.ascontiguousarray(C0)))
    D = tg.empty_colmajor(n, k, torch.float32, "cuda", ld=n + 2)
    fac = tg.factor_(A)
    tg.apply_qt_(fac, C, D)
    Q = to_dev(tg, A0)
    tg.tsqr_(Q)
    torch.cuda.synchronize()
    ref = to_host(Q).astype(np.float64).T @ C0.astype(np.float64)
    err = np.linalg.norm(to_host(D).astype(np.float64) - ref)
    assert err <= 20 * n * 2.0 ** -24 * np.linalg.norm(C0.astype(np.float64)), err
    tg.form_q_(fac)
    torch.cuda.synchronize()
    assert np.array_equal(to_host(A), to_host(Q))
