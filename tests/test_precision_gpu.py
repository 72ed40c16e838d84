"""GPU tests of the precision form (TSQR_PRECISION_TF32X3): FP32 tile
factorisation with FP64 norm/beta/tau, FP64 root combine, and every Q
assembly on the tcgen05 tensor cores in TF32 hi/lo three-product form.

Bar (the precision form's stated target): backward error and orthogonality
<= 1e-5 against the FP64 oracle, for every result; R within 1e-5 max|R| of
the FP64 oracle after diag(R) >= 0 on well-conditioned inputs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(tg, A):
    import torch
    m, n = A.shape
    d = tg.empty_colmajor(m, n, torch.float32, "cuda")
    d.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    return d


def to_host(x):
    return x.t().contiguous().cpu().numpy().T


def geometric_matrix(m, n, kappa, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.geomspace(1.0, 1.0 / kappa, n)
    return np.asfortranarray((U * s) @ V.T).astype(np.float32, order="F")


@pytest.mark.parametrize("m,n", [(27648, 32), (4096, 16), (100000, 64), (513, 32), (1000, 7), (40, 32),
                                 (300000, 48), (1, 1), (1024, 32)])
def test_precision_form_matches_oracle(orc, cuda, tg, m, n):
    A = orc.fill_uniform(m, n, np.float32, seed=4)
    dA = to_dev(tg, A)
    dR = tg.tsqr_(dA, precision="tf32x3")
    Q, R = to_host(dA), to_host(dR)
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met
    Qt, Rt = orc.householder_qr(A.astype(np.float64))
    Rs, Qs = np.asfortranarray(R.astype(np.float64)), np.asfortranarray(Q.astype(np.float64))
    orc.sign_fix(Qs, Rs)
    orc.sign_fix(Qt, Rt)
    assert np.abs(Rs - Rt).max() <= 1e-5 * np.abs(Rt).max()
    assert np.abs(Qs - Qt).max() <= 1e-5


@pytest.mark.parametrize("kappa", [1e3, 1e6])
def test_precision_form_ill_conditioned(orc, cuda, tg, kappa):
    A = geometric_matrix(200000, 32, kappa, 8)
    dA = to_dev(tg, A)
    dR = tg.tsqr_(dA, precision="tf32x3")
    met = orc.metrics(A, to_host(dA), to_host(dR))
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met


def test_precision_form_full_size(cuda, tg):
    import torch
    m, n = 4194304, 32
    g = torch.Generator(device="cuda").manual_seed(6)
    A0 = torch.rand((n, m), generator=g, device="cuda").mul_(2).sub_(1).t()
    A = A0.t().clone().t()
    R = tg.tsqr_(A, precision="tf32x3")
    torch.cuda.synchronize()
    E = A0.double() - A.double() @ R.double()
    back = (torch.linalg.norm(E) / torch.linalg.norm(A0.double())).item()
    G = A.double().t() @ A.double()
    orth = torch.linalg.norm(G - torch.eye(n, dtype=G.dtype, device=G.device)).item()
    assert back <= 1e-5 and orth <= 1e-5, (back, orth)


def test_precision_form_is_float_only(cuda, tg):
    import torch
    A = tg.empty_colmajor(1000, 8, torch.float64, "cuda").normal_()
    R = tg.tsqr_(A, precision="tf32x3")  # FP64 keeps the plain FP64 path (opts ignored)
    torch.cuda.synchronize()
    assert torch.isfinite(R).all()
