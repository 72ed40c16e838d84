"""GPU tests of the precision form (TSQR_PRECISION_TF32X3): the FP32 tile
factorisation on CUDA cores, and every Q assembly on the tcgen05 tensor
cores in TF32 hi/lo three-product form.

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
                                 (300000, 48), (1, 1), (1024, 32), (262144, 16), (70001, 13)])
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


@pytest.mark.parametrize("n", [32, 64])
@pytest.mark.parametrize("kappa", [1e3, 1e6])
def test_precision_form_ill_conditioned(orc, cuda, tg, kappa, n):
    A = geometric_matrix(200000, n, kappa, 8)
    dA = to_dev(tg, A)
    dR = tg.tsqr_(dA, precision="tf32x3")
    met = orc.metrics(A, to_host(dA), to_host(dR))
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met


@pytest.mark.parametrize("n", [32, 64])
def test_precision_form_full_size(cuda, tg, n):
    import torch
    m = 4194304
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


@pytest.mark.parametrize("m,n,reorth", [(27648, 128, False), (20000, 96, False), (50000, 256, True),
                                        (40000, 512, True), (30001, 520, False)])
def test_blocked_qr_precision_form(orc, cuda, tg, m, n, reorth):
    """qr with R12 = A1^T A2 and A2 -= A1 R12 in the precision form: the
    256-wide node's projection on the TMA-fed tcgen05 kernel (n = 512, 520),
    its update on tcgen05, the narrower products in FP32.  Bars: backward
    error <= 1e-5; orthogonality <= 1e-5 up to 256 columns, and the FP32
    bound 10 n u beyond (3.1e-4 at n = 512; block Gram-Schmidt's loss of
    orthogonality grows with n in FP32 arithmetic too)."""
    A = orc.fill_uniform(m, n, np.float32, seed=12)
    dA = to_dev(tg, A)
    dR = tg.qr_(dA, precision="tf32x3", reorth=reorth)
    met = orc.metrics(A, to_host(dA), to_host(dR))
    orth_bar = 1e-5 if n <= 256 else 10 * n * 2.0 ** -24
    assert met["backward"] <= 1e-5 and met["orth"] <= orth_bar, met


def test_blocked_qr_precision_matches_plain(orc, cuda, tg):
    A = orc.fill_uniform(27648, 128, np.float32, seed=13)
    outs = []
    for prec in ("plain", "tf32x3"):
        dA = to_dev(tg, A)
        dR = tg.qr_(dA, precision=prec)
        Q, R = np.asfortranarray(to_host(dA).astype(np.float64)), np.asfortranarray(to_host(dR).astype(np.float64))
        orc.sign_fix(Q, R)
        outs.append((Q, R))
    assert np.abs(outs[0][1] - outs[1][1]).max() <= 1e-5 * np.abs(outs[0][1]).max()
    assert np.abs(outs[0][0] - outs[1][0]).max() <= 1e-5


def test_blocked_qr_precision_large_kappa(cuda, tg):
    """131072 x 512, geometric singular values, condition 1e4, with one
    re-orthogonalisation pass.  Bar: backward error <= 1e-5 and
    orthogonality within the FP32 bound 10 n u (3.1e-4 at n = 512); the plain
    FP32 form is measured beside it on the same input (measured on GB300:
    plain 3.0e-7 / 3.6e-5, precision 2.0e-6 / 1.9e-5)."""
    import torch
    m, n = 131072, 512
    g = torch.Generator(device="cuda").manual_seed(3)
    U, _ = torch.linalg.qr(torch.randn(m, n, generator=g, device="cuda", dtype=torch.float64))
    V, _ = torch.linalg.qr(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64))
    s = torch.logspace(0, -4, n, device="cuda", dtype=torch.float64)
    A0 = ((U * s) @ V.t()).float()
    figs = {}
    for prec in ("plain", "tf32x3"):
        A = A0.t().contiguous().t()
        R = tg.qr_(A, precision=prec, reorth=True)
        torch.cuda.synchronize()
        E = A0.double() - A.double() @ R.double()
        back = (torch.linalg.norm(E) / torch.linalg.norm(A0.double())).item()
        G = A.double().t() @ A.double()
        orth = torch.linalg.norm(G - torch.eye(n, dtype=G.dtype, device=G.device)).item()
        figs[prec] = (back, orth)
    u = 2.0 ** -24
    for back, orth in figs.values():
        assert back <= 1e-5 and orth <= 10 * n * u, figs


def test_workspace_status_word_is_clear_after_tensor_core_calls(orc, cuda, tg):
    """The tcgen05 kernels' bounded mbarrier waits report a timeout through
    the status word at the start of the workspace; after ordinary calls of
    every precision-form entry point it must read clear."""
    import torch
    m, n = 70000, 32
    A = orc.fill_uniform(m, n, np.float32, seed=9)
    dA = to_dev(tg, A)
    nb = tg.workspace_bytes(m, n, torch.float32, precision="tf32x3")
    w = torch.full((nb,), 0xFF, dtype=torch.uint8, device="cuda")  # the call must clear the word itself
    tg.tsqr_(dA, precision="tf32x3", work=w)
    torch.cuda.synchronize()
    assert tg.lib().tsqr_workspace_check(w.data_ptr()) == 0
    m2, n2 = 20000, 256
    B = to_dev(tg, orc.fill_uniform(m2, n2, np.float32, seed=10))
    nb2 = tg.qr_workspace_bytes(m2, n2, torch.float32, precision="tf32x3")
    w2 = torch.full((nb2,), 0xFF, dtype=torch.uint8, device="cuda")
    tg.qr_(B, precision="tf32x3", work=w2)
    torch.cuda.synchronize()
    assert tg.lib().tsqr_workspace_check(w2.data_ptr()) == 0
    hA = torch.from_numpy(np.ascontiguousarray(A.T)).pin_memory().t()
    o = tg._opts("tf32x3")
    import ctypes
    nb3 = int(tg.lib().tsqr_host_workspace_bytes(m, n, 4, ctypes.byref(o)))
    w3 = torch.full((nb3,), 0xFF, dtype=torch.uint8, device="cuda")
    tg.tsqr_host_(hA, precision="tf32x3", work=w3)
    torch.cuda.synchronize()
    assert tg.lib().tsqr_workspace_check(w3.data_ptr()) == 0


def test_a_tensor_core_wait_that_runs_out_is_reported_and_the_next_call_succeeds(orc, cuda, tg):
    """Failure detection of the tcgen05 kernels, made to happen on purpose:
    with their MMA waits limited to 0 polls (tsqr_debug_set_wait_limit), the
    first wait of every tensor-core kernel gives up; the kernel lets its
    in-flight MMAs retire (that wait keeps the full limit), frees its TMEM and
    returns, and the call's status word reads TSQR_ERR_CUDA.  Nothing is left
    broken: with the default limit restored the same calls succeed, clear the
    word and meet the form's bar (backward <= 1e-5; orthogonality <= 1e-5
    for TSQR, 10 n u for the 512-column QR)."""
    import torch
    L = tg.lib()
    m, n = 70000, 32
    A = orc.fill_uniform(m, n, np.float32, seed=21)
    m2, n2 = 20000, 512  # the 256-wide node: TMA-fed tcgen05 projection and tcgen05 update
    B = orc.fill_uniform(m2, n2, np.float32, seed=22)
    w = torch.zeros(tg.workspace_bytes(m, n, torch.float32, precision="tf32x3"), dtype=torch.uint8, device="cuda")
    w2 = torch.zeros(tg.qr_workspace_bytes(m2, n2, torch.float32, precision="tf32x3"), dtype=torch.uint8,
                     device="cuda")
    try:
        assert L.tsqr_debug_set_wait_limit(0) == 0
        tg.tsqr_(to_dev(tg, A), precision="tf32x3", work=w)        # tc_apply_tiles
        tg.qr_(to_dev(tg, B), precision="tf32x3", work=w2)         # tc_tn_tma_kernel, tc_gemm_kernel
        torch.cuda.synchronize()
        assert L.tsqr_workspace_check(w.data_ptr()) == 4           # TSQR_ERR_CUDA
        assert L.tsqr_workspace_check(w2.data_ptr()) == 4
    finally:
        L.tsqr_debug_set_wait_limit(-1)
    torch.cuda.synchronize()                                        # the context is still usable
    dA, dB = to_dev(tg, A), to_dev(tg, B)
    dR = tg.tsqr_(dA, precision="tf32x3", work=w)
    dR2 = tg.qr_(dB, precision="tf32x3", work=w2)
    torch.cuda.synchronize()
    assert L.tsqr_workspace_check(w.data_ptr()) == 0
    assert L.tsqr_workspace_check(w2.data_ptr()) == 0
    # the 512-column block Gram-Schmidt QR: orthogonality within the FP32
    # bound 10 n u (3.1e-4)
    for M0, dQ, dRr, orth_bar in ((A, dA, dR, 1e-5), (B, dB, dR2, 10 * n2 * 2.0 ** -24)):
        met = orc.metrics(M0, to_host(dQ), to_host(dRr))
        assert met["backward"] <= 1e-5 and met["orth"] <= orth_bar, met


@pytest.mark.parametrize("m,n", [(27648, 32), (100000, 64), (70001, 13), (1000, 7), (300000, 16)])
def test_fp64_scalars_option(orc, cuda, tg, m, n):
    """tsqr_opts.fp64_scalars: each column's Householder norm, beta and tau in
    FP64 inside the FP32 tile factorisation.  Same bar as the form; R agrees
    with the default form's to the form's precision."""
    A = orc.fill_uniform(m, n, np.float32, seed=31)
    dA = to_dev(tg, A)
    dR = tg.tsqr_(dA, precision="tf32x3", fp64_scalars=True)
    dA0 = to_dev(tg, A)
    dR0 = tg.tsqr_(dA0, precision="tf32x3")
    Q, R = to_host(dA), to_host(dR)
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met
    R0 = to_host(dR0)
    assert np.abs(R - R0).max() <= 1e-5 * np.abs(R0).max()


@pytest.mark.parametrize("m,n", [(300000, 32), (27648, 32), (500, 20), (70001, 13)])
def test_fp64_root_option(orc, cuda, tg, m, n):
    """tsqr_opts.fp64_root: the root of the tree factored by the FP64 tree
    (a single-tile problem: the whole of A).  Same bar as the form."""
    A = orc.fill_uniform(m, n, np.float32, seed=32)
    dA = to_dev(tg, A)
    dR = tg.tsqr_(dA, precision="tf32x3", fp64_root=True)
    met = orc.metrics(A, to_host(dA), to_host(dR))
    assert met["backward"] <= 1e-5 and met["orth"] <= 1e-5, met
    with pytest.raises(tg.TsqrError):
        tg.tsqr_(to_dev(tg, orc.fill_uniform(1000, 48, np.float32, seed=1)), precision="tf32x3", fp64_root=True)


@pytest.mark.parametrize("form,dtype,m,n", [("plain", np.float32, 27648, 32), ("plain", np.float32, 70001, 13),
                                            ("plain", np.float64, 27648, 32), ("tf32x3", np.float32, 100000, 32),
                                            ("tf32x3", np.float32, 300, 20)])
def test_tsqr_reorthogonalisation_pass(orc, cuda, tg, form, dtype, m, n):
    """tsqr_opts.reorth for TSQR: a second TSQR of the computed Q, R <- R2 R1.
    The result meets the form's bar (plain: 10 n u; tf32x3: 1e-5), and R
    agrees with the single pass's R (R2 is the identity to rounding)."""
    import torch
    A = orc.fill_uniform(m, n, dtype, seed=33)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    dA = tg.empty_colmajor(m, n, tdt, "cuda")
    dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    w = torch.zeros(tg.workspace_bytes(m, n, tdt, precision=form, reorth=True), dtype=torch.uint8, device="cuda")
    assert w.numel() > tg.workspace_bytes(m, n, tdt, precision=form)
    dR = tg.tsqr_(dA, precision=form, reorth=True, work=w)
    torch.cuda.synchronize()
    Q, R = to_host(dA), to_host(dR)
    met = orc.metrics(A, Q, R)
    u = orc.unit_roundoff(dtype)
    bar = 1e-5 if form == "tf32x3" else 10 * n * u
    assert met["backward"] <= bar and met["orth"] <= bar, met
    assert np.all(np.tril(R, -1) == 0)
    dA1 = tg.empty_colmajor(m, n, tdt, "cuda")
    dA1.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    R1 = to_host(tg.tsqr_(dA1, precision=form))
    tol = 1e-5 if form == "tf32x3" else 100 * n * u
    assert np.abs(R - R1).max() <= tol * np.abs(R1).max()
    if form == "tf32x3":
        assert tg.lib().tsqr_workspace_check(w.data_ptr()) == 0


@pytest.mark.parametrize("algorithm", ["block_gs", "householder"])
def test_bf16x3_blocked_qr(orc, cuda, tg, algorithm):
    """TSQR_PRECISION_BF16X3 for qr: the GEMMs on tcgen05 with BF16 hi/lo
    three-product splits (each product carries about 2^-16 relative error,
    against 2^-21 for TF32x3); the TSQR panels run TF32x3.  Bar: backward
    error <= 1e-5 against FP64, orthogonality <= 5e-4 (block Gram-Schmidt on
    a standard-normal matrix; the Householder algorithm stays near 1e-5), and
    R within 1e-4 max|R| of the TF32x3 form's."""
    import torch
    m, n = 27648, 128
    rng = np.random.default_rng(129)
    A = np.asfortranarray(rng.standard_normal((m, n)).astype(np.float32))
    out = {}
    for prec in ("bf16x3", "tf32x3"):
        dA = to_dev(tg, A)
        w = torch.zeros(tg.qr_workspace_bytes(m, n, torch.float32, precision=prec, algorithm=algorithm),
                        dtype=torch.uint8, device="cuda")
        dR = tg.qr_(dA, precision=prec, algorithm=algorithm, work=w)
        torch.cuda.synchronize()
        assert tg.lib().tsqr_workspace_check(w.data_ptr()) == 0
        out[prec] = (to_host(dA), to_host(dR))
    Q, R = out["bf16x3"]
    met = orc.metrics(A, Q, R)
    orth_bar = 5e-4 if algorithm == "block_gs" else 1e-4
    assert met["backward"] <= 1e-5 and met["orth"] <= orth_bar, met
    R32 = out["tf32x3"][1]
    Rs, R32s = np.asfortranarray(R.astype(np.float64)), np.asfortranarray(R32.astype(np.float64))
    Qs, Q32s = np.asfortranarray(Q.astype(np.float64)), np.asfortranarray(out["tf32x3"][0].astype(np.float64))
    orc.sign_fix(Qs, Rs)
    orc.sign_fix(Q32s, R32s)
    assert np.abs(Rs - R32s).max() <= 1e-4 * np.abs(R32s).max()
