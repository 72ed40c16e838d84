"""tsqr_s_noalloc: FP32 TSQR for callers that cannot allocate device memory.

Such callers include frameworks that have reserved nearly all device memory
for their own pool, programs working to a fixed memory budget, and code that
cannot afford the synchronisation a cudaFree may cause.  The entry point
keeps its tree workspace in a static device array inside the library instead
of asking for one.  It is checked here through the C ABI against the
ordinary entry point (tsqr_s_ex, plain precision) on two calls in a row.  Both
run the same kernels over the same level layout, so Q and R must agree bit
for bit; the oracle's backward error and orthogonality must also meet the
plain-form bar (10 n u, u = 2^-24).  The second call uses a different shape,
so it runs over scratch contents left by the first.  A further check reads the
device's free memory around a call: it must not change.

The file name sorts last so that pytest collects it after every other test: a
run that stops at its first failure (-x) has then already run all the rest.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(tg):
    fn = tg.lib().tsqr_s_noalloc
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.c_int64, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _dev(tg, A):
    import torch
    m, n = A.shape
    d = tg.empty_colmajor(m, n, torch.float32, "cuda")
    d.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    return d


def _host(x):
    return x.t().contiguous().cpu().numpy().T


def test_noalloc_matches_ordinary_entry_point_on_two_calls(orc, cuda, tg):
    import torch
    fn = _noalloc(tg)
    u = 2.0 ** -24
    for call, (m, n, seed) in enumerate([(300000, 32, 1), (120000, 24, 2)]):
        A = orc.fill_uniform(m, n, np.float32, seed=seed)
        dA_ref = _dev(tg, A)
        dR_ref = tg.tsqr_(dA_ref)
        dA = _dev(tg, A)
        dR = tg.empty_colmajor(n, n, torch.float32, "cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = fn(m, n, dA.data_ptr(), m, dR.data_ptr(), n, stream)
        assert rc == 0, (call, rc, tg.lib().tsqr_status_string(rc))
        torch.cuda.synchronize()
        Q, R = _host(dA), _host(dR)
        Qr, Rr = _host(dA_ref), _host(dR_ref)
        assert np.array_equal(R, Rr), (call, np.abs(R - Rr).max())
        assert np.array_equal(Q, Qr), (call, np.abs(Q - Qr).max())
        met = orc.metrics(A, Q, R)
        assert met["backward"] <= 10 * n * u and met["orth"] <= 10 * n * u, (call, met)


def test_noalloc_call_leaves_free_device_memory_unchanged(orc, cuda, tg):
    """After a first call (which sets up the scratch address), a call takes
    no device memory: cudaMemGetInfo reads the same before and after."""
    import torch
    fn = _noalloc(tg)
    m, n = 200000, 32
    A = orc.fill_uniform(m, n, np.float32, seed=3)
    dA = _dev(tg, A)
    dR = tg.empty_colmajor(n, n, torch.float32, "cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert fn(m, n, dA.data_ptr(), m, dR.data_ptr(), n, stream) == 0
    torch.cuda.synchronize()
    dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert fn(m, n, dA.data_ptr(), m, dR.data_ptr(), n, stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda, tg):
    fn = _noalloc(tg)
    fake = ctypes.c_void_p(0x1000)
    m = 8 * 1024 * 1024  # its tree workspace is larger than the static scratch
    assert tg.workspace_bytes(m, 32, "float32") > 16 << 20
    assert fn(m, 32, fake, m, fake, 32, None) == 3  # TSQR_ERR_WORKSPACE, nothing launched
