"""GPU tests of the batched form (tsqr_batched_s): many independent FP32
problems of uneven heights and widths factored by one short sequence of
launches, which can be captured into a CUDA graph.

Bar: every problem meets the plain-path parity bar (backward error and
orthogonality <= 10 n u, u = 2^-24) and matches the single-problem entry
point on the same input to 1e-6 (same tree, same tile heights).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(tg, A):
    import torch
    m, n = A.shape
    d = tg.empty_colmajor(m, n, torch.float32, "cuda")
    d.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    return d


def host(x):
    return x.t().contiguous().cpu().numpy().T


SHAPES = [(1, 1), (5, 3), (64, 64), (100, 8), (513, 32), (2000, 17), (4096, 16), (20000, 32), (3000, 64),
          (70000, 33), (129, 1), (1025, 8), (8192, 64), (6000, 24), (40000, 16), (700, 48)]


def test_batch_matches_single_calls_and_oracle(orc, cuda, tg):
    import torch
    As = [orc.fill_uniform(m, n, np.float32, seed=100 + k) for k, (m, n) in enumerate(SHAPES)]
    dAs = [dev(tg, A) for A in As]
    dRs = tg.tsqr_batched_(dAs)
    torch.cuda.synchronize()
    u = 2.0 ** -24
    for A, dA, dR in zip(As, dAs, dRs):
        m, n = A.shape
        Q, R = host(dA), host(dR)
        met = orc.metrics(A, Q, R)
        assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, (m, n, met)
        sA = dev(tg, A)
        sR = tg.tsqr_(sA)
        assert np.abs(host(sR) - R).max() <= 1e-6 * np.abs(R).max(), (m, n)
        assert np.abs(host(sA) - Q).max() <= 1e-6, (m, n)


def test_batch_replays_from_a_cuda_graph(orc, cuda, tg):
    import torch
    shapes = [(3000, 32), (500, 8), (10000, 16), (2500, 64)]
    As = [orc.fill_uniform(m, n, np.float32, seed=7 + k) for k, (m, n) in enumerate(shapes)]
    dAs = [dev(tg, A) for A in As]
    Rs = [tg.empty_colmajor(n, n, torch.float32, "cuda") for _, n in shapes]
    m_ = [a.shape[0] for a in As]
    n_ = [a.shape[1] for a in As]
    import ctypes
    c = len(shapes)
    nbytes = tg.lib().tsqr_batched_workspace_bytes(c, (ctypes.c_int64 * c)(*m_), (ctypes.c_int64 * c)(*n_))
    work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        tg.tsqr_batched_(dAs, Rs, work=work, stream=s)  # warm-up outside capture
    s.synchronize()
    for dA, A in zip(dAs, As):
        dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        tg.tsqr_batched_(dAs, Rs, work=work, stream=s)
    for _ in range(2):  # replay twice on fresh inputs
        for dA, A in zip(dAs, As):
            dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
        g.replay()
        torch.cuda.synchronize()
        for A, dA, R in zip(As, dAs, Rs):
            n = A.shape[1]
            met = orc.metrics(A, host(dA), host(R))
            assert met["backward"] <= 10 * n * 2.0 ** -24 and met["orth"] <= 10 * n * 2.0 ** -24, met


def test_uneven_512_batch(cuda, tg):
    """512 problems: heights log-uniform in [2048, 262144], widths from
    {8, 16, 32, 64}, entries uniform[-1, 1), seeded."""
    import torch
    rng = np.random.default_rng(2024)
    ms = np.exp(rng.uniform(np.log(2048), np.log(262144), 512)).astype(np.int64)
    ns = rng.choice([8, 16, 32, 64], 512)
    g = torch.Generator(device="cuda").manual_seed(1)
    A0 = [torch.rand((int(n), int(m)), generator=g, device="cuda").mul_(2).sub_(1).t() for m, n in zip(ms, ns)]
    As = [a.t().clone().t() for a in A0]
    Rs = tg.tsqr_batched_(As)
    torch.cuda.synchronize()
    for k in range(0, 512, 37):
        a0, q, r = A0[k].double(), As[k].double(), Rs[k].double()
        n = a0.shape[1]
        back = (torch.linalg.norm(a0 - q @ r) / torch.linalg.norm(a0)).item()
        orth = torch.linalg.norm(q.t() @ q - torch.eye(n, dtype=q.dtype, device=q.device)).item()
        assert back <= 10 * n * 2.0 ** -24 and orth <= 10 * n * 2.0 ** -24, (k, back, orth)


def test_batch_argument_checks(cuda, tg):
    import ctypes
    L = tg.lib()
    one = (ctypes.c_int64 * 1)
    p = (ctypes.c_void_p * 1)(0x1000)
    assert L.tsqr_batched_s(0, None, None, None, None, None, None, None, 0, None, None) == 0
    assert L.tsqr_batched_s(1, p, one(100), one(65), one(100), p, one(65), p, 1 << 20, None, None) == 2
    assert L.tsqr_batched_s(1, p, one(10), one(20), one(10), p, one(20), p, 1 << 20, None, None) == 1
    assert L.tsqr_batched_s(1, p, one(100), one(8), one(100), p, one(8), p, 1, None, None) == 3


def _set_all(tg, cand):
    for c in range(4):
        for b in range(3):
            assert tg.lib().tsqr_batched_set_choice(c, b, cand) == 0


@pytest.mark.parametrize("cand", [0, 1])
def test_every_tuning_candidate_meets_the_bar(orc, cuda, tg, cand):
    """Each candidate tile configuration of the autotuner, forced for every
    class and bucket, meets the plain-path parity bar (its tree differs from
    the single-problem path's when the tile height differs)."""
    import torch
    _set_all(tg, cand)
    try:
        As = [orc.fill_uniform(m, n, np.float32, seed=300 + k) for k, (m, n) in enumerate(SHAPES)]
        dAs = [dev(tg, A) for A in As]
        dRs = tg.tsqr_batched_(dAs)
        torch.cuda.synchronize()
        u = 2.0 ** -24
        for A, dA, dR in zip(As, dAs, dRs):
            m, n = A.shape
            met = orc.metrics(A, host(dA), host(dR))
            assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, (cand, m, n, met)
    finally:
        _set_all(tg, 0)


def test_tuner_picks_valid_candidates_and_results_hold(orc, cuda, tg):
    import torch
    shapes = [(2048, 8), (5000, 16), (30000, 32), (100000, 64), (70000, 16), (3000, 32)]
    try:
        table = tg.batched_tune_(shapes, reps=2)
        for (c, b), (k, rows) in table.items():
            assert k in (0, 1) and rows == tg.lib().tsqr_batched_candidate_rows(c, k)
        As = [orc.fill_uniform(m, n, np.float32, seed=400 + k) for k, (m, n) in enumerate(shapes)]
        dAs = [dev(tg, A) for A in As]
        dRs = tg.tsqr_batched_(dAs)
        torch.cuda.synchronize()
        u = 2.0 ** -24
        for A, dA, dR in zip(As, dAs, dRs):
            m, n = A.shape
            met = orc.metrics(A, host(dA), host(dR))
            assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, (m, n, met)
    finally:
        _set_all(tg, 0)
