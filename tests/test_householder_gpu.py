"""GPU tests of the blocked Householder QR (qr_*_ex with algorithm
TSQR_QR_HOUSEHOLDER): TSQR panels, Householder vectors reconstructed from
each panel's Q, compact-WY trailing updates, Q accumulated backwards.  Not
in the reference, whose qr<T> is block Gram-Schmidt (block_QR.h:72-95).

Bars (u = 2^-24 / 2^-53):
  * against the FP64 oracle's Householder QR, after normalising
    diag(R) >= 0: max |dR| <= 100 n u max|R| and max |dQ| <= 100 n u on
    well-conditioned inputs;
  * backward error and orthogonality <= 10 n u for any condition number
    (cond 1e6 in FP32, 1e12 in FP64), where the block Gram-Schmidt path
    loses orthogonality in proportion to the condition number;
  * the TF32X3 form: both figures <= 1e-5.
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


def conditioned(m, n, kappa, dtype, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    sig = np.logspace(0, -np.log10(kappa), n)
    return ((U * sig) @ V.T).astype(dtype)


def factor(tg, A0, **kw):
    import torch
    Q = to_dev(tg, A0)
    R = tg.qr_(Q, **kw)
    torch.cuda.synchronize()
    return to_host(Q), to_host(R)


@pytest.mark.parametrize("m,n,dtype", [(27648, 128, np.float32), (4096, 64, np.float32),
                                       (10000, 100, np.float32), (8192, 96, np.float64),
                                       (3000, 40, np.float64)])
def test_householder_matches_oracle(orc, cuda, tg, m, n, dtype):
    A0 = orc.fill_uniform(m, n, dtype, seed=61)
    Q, R = factor(tg, A0, algorithm="householder")
    u = orc.unit_roundoff(dtype)
    met = orc.metrics(A0, Q, R)
    assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, met
    assert np.all(R[np.tril_indices(n, -1)] == 0)
    Qt, Rt = orc.householder_qr(A0.astype(np.float64))
    Qs, Rs = Q.astype(np.float64), R.astype(np.float64)
    orc.sign_fix(Qs, Rs)
    orc.sign_fix(Qt, Rt)
    assert np.abs(Rs - Rt).max() <= 100 * n * u * np.abs(Rt).max()
    assert np.abs(Qs - Qt).max() <= 100 * n * u


@pytest.mark.parametrize("m,n,dtype,kappa", [(20000, 128, np.float32, 1e6), (8192, 64, np.float64, 1e12)])
def test_householder_stays_orthogonal_when_ill_conditioned(orc, cuda, tg, m, n, dtype, kappa):
    A0 = conditioned(m, n, kappa, dtype, seed=62)
    u = orc.unit_roundoff(dtype)
    Qh, Rh = factor(tg, A0, algorithm="householder")
    hh = orc.metrics(A0, Qh, Rh)
    assert hh["backward"] <= 10 * n * u and hh["orth"] <= 10 * n * u, hh
    # the reference's algorithm on the same input, for contrast
    Qg, Rg = factor(tg, A0)
    gs = orc.metrics(A0, Qg, Rg)
    assert gs["orth"] > 100 * hh["orth"], (gs, hh)


def test_householder_precision_form(orc, cuda, tg):
    m, n = 65536, 256
    A0 = conditioned(m, n, 1e4, np.float32, seed=63)
    Q, R = factor(tg, A0, algorithm="householder", precision="tf32x3")
    met = orc.metrics(A0, Q, R)
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met


def test_householder_rejects_wide_panels(cuda, tg):
    import torch
    A = tg.empty_colmajor(1000, 100, torch.float32, "cuda")
    with pytest.raises(tg.TsqrError):
        tg.qr_(A, algorithm="householder", panel=64)


def test_householder_with_padded_leading_dimensions(orc, cuda, tg):
    import torch
    m, n = 9000, 70
    A0 = orc.fill_uniform(m, n, np.float32, seed=64)
    A = tg.empty_colmajor(m, n, torch.float32, "cuda", ld=m + 7)
    A.copy_(torch.from_numpy(np.ascontiguousarray(A0)))
    R = tg.empty_colmajor(n, n, torch.float32, "cuda", ld=n + 3)
    tg.qr_(A, R, algorithm="householder")
    torch.cuda.synchronize()
    met = orc.metrics(A0, to_host(A), to_host(R))
    u = 2.0 ** -24
    assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, met
