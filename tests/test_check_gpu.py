"""GPU tests of the device accuracy check tsqr_check (check_ in Python),
which replaces the reference's host accuracy check check_QR_accuracy
(utils.h:317-455).

Bar: its four figures equal the FP64 oracle's (orc.metrics) on the same
factorisation -- Frobenius figures within 1e-6 relative, spectral ones
(largest eigenvalues by Jacobi on both sides) within 1e-4 relative, for
FP64 inputs also within 4 sqrt(m) n u64 absolute -- and
its element gate (the reference's all_close, utils.h:148-174) reports
exactly the planted failures, the first one in column-major order.
Mistakes are planted in host copies of Q (numpy) before upload.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(tg, A_np):
    import torch
    m, n = A_np.shape
    dt = torch.float32 if A_np.dtype == np.float32 else torch.float64
    A = tg.empty_colmajor(m, n, dt, "cuda")
    A.copy_(torch.from_numpy(np.ascontiguousarray(A_np)))
    return A


def to_host(x):
    return x.t().contiguous().cpu().numpy().T


def close(a, b, rtol, atol=1e-300):
    return abs(a - b) <= atol + rtol * abs(b)


@pytest.mark.parametrize("kind,m,n,dtype,precision", [
    ("tsqr", 27648, 32, np.float32, "plain"),
    ("tsqr", 100000, 32, np.float32, "tf32x3"),  # past the reference check's m = 46,340 limit
    ("tsqr", 1000, 13, np.float64, "plain"),
    ("tsqr", 70001, 64, np.float32, "plain"),
    ("qr", 27648, 128, np.float32, "plain"),
    ("qr", 8192, 128, np.float64, "plain"),
])
def test_figures_match_oracle(orc, cuda, tg, kind, m, n, dtype, precision):
    import torch
    A0 = orc.fill_uniform(m, n, dtype, seed=41)
    dA0 = to_dev(tg, A0)
    Q = dA0.t().clone().t()
    R = (tg.tsqr_ if kind == "tsqr" else tg.qr_)(Q, precision=precision)
    torch.cuda.synchronize()
    res = tg.check_(dA0, Q, R)
    met = orc.metrics(A0, to_host(Q), to_host(R))
    assert res["gate_failures"] == 0 and res["first_row"] is None, res
    # FP64 inputs: the figures (~1e-15) are at the rounding level of forming
    # the Gram matrices in FP64 (about sqrt(m) u64 per entry), so two FP64
    # implementations agree only to that absolute level
    atol = 4 * np.sqrt(m) * n * 2.0 ** -53 if dtype == np.float64 else 1e-300
    assert close(res["backward_fro"], met["backward"], 1e-6, atol), (res, met)
    assert close(res["orth_fro"], met["orth"], 1e-6, atol), (res, met)
    assert close(res["backward_2"], met["backward_2"], 1e-4, atol), (res, met)
    assert close(res["orth_2"], met["orth_2_n"], 1e-4, atol), (res, met)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gate_reports_planted_errors(orc, cuda, tg, dtype):
    import torch
    m, n = 5000, 24
    A0 = orc.fill_uniform(m, n, dtype, seed=42)
    dA0 = to_dev(tg, A0)
    Q = dA0.t().clone().t()
    R = tg.tsqr_(Q)
    torch.cuda.synchronize()
    Qh, Rh = to_host(Q), to_host(R)
    # two wrong elements: column 3 row 4000 and column 7 row 10 (the later
    # one in column-major order is planted first)
    Qbad = Qh.copy()
    Qbad[10, 7] += 0.5
    Qbad[4000, 3] -= 0.25
    res = tg.check_(dA0, to_dev(tg, Qbad), R)
    assert res["gate_failures"] >= 2
    assert (res["first_row"], res["first_col"]) == (4000, 3)
    qr_val = float(np.dot(Qbad[4000].astype(np.float64), Rh[:, 3].astype(np.float64)))
    assert abs(res["first_value"] - qr_val) <= 1e-6 * max(1.0, abs(qr_val))
    assert res["first_ref"] == float(A0[4000, 3])
    # a tolerance wide enough for the planted errors lets every element pass
    wide = tg.check_(dA0, to_dev(tg, Qbad), R, atol=1e6, rtol=0.0)
    assert wide["gate_failures"] == 0


def test_gate_counts_nan(orc, cuda, tg):
    import torch
    m, n = 3000, 16
    A0 = orc.fill_uniform(m, n, np.float32, seed=43)
    dA0 = to_dev(tg, A0)
    Q = dA0.t().clone().t()
    R = tg.tsqr_(Q)
    torch.cuda.synchronize()
    Qbad = to_host(Q).copy()
    Qbad[123, 0] = np.nan
    res = tg.check_(dA0, to_dev(tg, Qbad), R)
    # row 123 of QR is NaN in every column
    assert res["gate_failures"] == n
    assert (res["first_row"], res["first_col"]) == (123, 0)


def test_check_rejects_bad_arguments(cuda, tg):
    import ctypes
    import torch
    L = tg.lib()
    a = torch.zeros((8, 100), dtype=torch.float32, device="cuda")
    r = torch.zeros((8, 8), dtype=torch.float32, device="cuda")
    w = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    res = tg.CheckResult()
    call = lambda eb, m, n, lda, ldr, wb: L.tsqr_check(eb, m, n, a.data_ptr(), lda, a.data_ptr(), lda, r.data_ptr(),
                                                       ldr, 1e-4, 1e-5, w.data_ptr(), wb, None, ctypes.byref(res))
    assert call(4, 100, 8, 99, 8, 1 << 20) == 1   # lda < m
    assert call(4, 100, 8, 100, 7, 1 << 20) == 1  # ldr < n
    assert call(2, 100, 8, 100, 8, 1 << 20) == 1  # element size
    assert call(4, 100, 8, 100, 8, 64) == 3       # workspace too small
    assert call(4, 100, 8, 100, 8, 1 << 20) == 0


def test_check_with_padded_leading_dimensions(orc, cuda, tg):
    import torch
    m, n = 20000, 20
    A0 = orc.fill_uniform(m, n, np.float64, seed=44)
    dA0 = tg.empty_colmajor(m, n, torch.float64, "cuda", ld=m + 3)
    dA0.copy_(torch.from_numpy(np.ascontiguousarray(A0)))
    Q = tg.empty_colmajor(m, n, torch.float64, "cuda", ld=m + 9)
    Q.copy_(dA0)
    R = tg.empty_colmajor(n, n, torch.float64, "cuda", ld=n + 4)
    tg.tsqr_(Q, R)
    torch.cuda.synchronize()
    res = tg.check_(dA0, Q, R)
    met = orc.metrics(A0, to_host(Q), to_host(R))
    atol = 4 * np.sqrt(m) * n * 2.0 ** -53
    assert res["gate_failures"] == 0
    assert close(res["backward_fro"], met["backward"], 1e-6, atol) and close(res["orth_fro"], met["orth"], 1e-6, atol)
