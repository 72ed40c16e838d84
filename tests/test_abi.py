"""CPU tests of the drop-in boundary: the C-ABI library loads, exports every
symbol include/tsqr_gb300.h declares, and rejects bad arguments before any
CUDA call (the reference asserts or prints instead: TallShinnyQR.h:92-109,
block_QR.h:78-79).  No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tsqr_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_][a-z0-9_]*\s*\*?\s+([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for n in ("tsqr_float", "tsqr_double", "qr_float", "qr_double", "tsqr_s_ex", "tsqr_d_ex", "qr_s_ex",
              "qr_d_ex", "tsqr_workspace_bytes", "qr_workspace_bytes", "tsqr_batched_s", "tsqr_status_string"):
        assert n in names


def test_library_exports_every_declared_symbol(tg):
    L = ctypes.CDLL(tg.library_path())
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(tg.EXPORTS)


def test_status_strings(tg):
    for s in range(6):
        assert tg.lib().tsqr_status_string(s)
    assert tg.lib().tsqr_version().decode().count(".") == 2


@pytest.mark.parametrize("m,n,lda,ldr,st", [
    (0, 1, 1, 1, 1), (10, 0, 10, 1, 1), (10, 20, 10, 20, 1),   # m < n rejected (TallShinnyQR.h:92)
    (100, 8, 99, 8, 1), (100, 8, 100, 7, 1), (100, 65, 100, 65, 2),
])
def test_tsqr_argument_checks_need_no_gpu(tg, m, n, lda, ldr, st):
    o = tg.Opts()
    fake = ctypes.c_void_p(0x1000)
    rc = tg.lib().tsqr_s_ex(m, n, fake, lda, fake, ldr, fake, 1 << 20, ctypes.byref(o), None)
    assert rc == st


def test_null_pointers_and_options_rejected(tg):
    o = tg.Opts()
    fake = ctypes.c_void_p(0x1000)
    L = tg.lib()
    assert L.tsqr_s_ex(64, 8, None, 64, fake, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    assert L.tsqr_d_ex(64, 8, fake, 64, None, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    o.reserved[0] = 7
    assert L.qr_s_ex(64, 8, fake, 64, fake, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    o = tg.Opts()
    o.precision = 9
    assert L.tsqr_s_ex(64, 8, fake, 64, fake, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    assert L.tsqr_d_ex(64, 33, fake, 64, fake, 33, fake, 1 << 20, None, None) == 2  # FP64 n <= 32


def test_workspace_too_small_is_reported(tg):
    o = tg.Opts()
    fake = ctypes.c_void_p(0x1000)
    need = tg.lib().tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(o))
    assert need > 0
    assert tg.lib().tsqr_s_ex(1 << 20, 32, fake, 1 << 20, fake, 32, fake, need - 1, ctypes.byref(o), None) == 3
    assert tg.lib().tsqr_s_ex(1 << 20, 32, fake, 1 << 20, fake, 32, None, need, ctypes.byref(o), None) == 3


def test_workspace_sizes_are_small(tg):
    # The R stack of the tree is the only workspace: n/B of A per level.
    for n in (8, 16, 32, 64):
        m = 4194304
        ws = tg.workspace_bytes(m, n, "float32")
        assert 0 < ws < 0.35 * m * n * 4
    assert tg.workspace_bytes(100, 200, "float32") == 0        # m < n
    assert tg.qr_workspace_bytes(27648, 128, "float64") > 0
    assert tg.qr_workspace_bytes(27648, 128, "float64", reorth=True) > tg.qr_workspace_bytes(27648, 128, "float64")


def test_host_entry_argument_checks_need_no_gpu(tg):
    """tsqr_s_host / tsqr_d_host reject bad sizes, leading dimensions,
    options and workspaces before any CUDA call."""
    L = tg.lib()
    a = (ctypes.c_float * 400)()
    q = (ctypes.c_float * 400)()
    r = (ctypes.c_float * 16)()
    o = tg._opts("plain")
    p = lambda x: ctypes.cast(x, ctypes.c_void_p)

    def call(m, n, lda, ldq, ldr, work=1, nbytes=1 << 30, opts=o, fn=L.tsqr_s_host):
        return fn(m, n, p(a), lda, p(q), ldq, p(r), ldr, ctypes.c_void_p(work), nbytes, ctypes.byref(opts), None)

    assert call(100, 4, 99, 100, 4) == 1    # lda < m
    assert call(100, 4, 100, 99, 4) == 1    # ldq < m
    assert call(100, 4, 100, 100, 3) == 1   # ldr < n
    assert call(3, 4, 100, 100, 4) == 1     # m < n
    assert call(100, 65, 100, 100, 65) == 2  # n above the FP32 limit
    assert call(100, 4, 100, 100, 4, work=0) == 3
    assert call(100, 4, 100, 100, 4, nbytes=16) == 3
    assert call(100, 4, 100, 100, 4, opts=tg._opts("bf16x3")) == 2
    assert call(100, 4, 100, 100, 4, opts=tg._opts("tf32x3"), fn=L.tsqr_d_host) == 2
    assert L.tsqr_host_workspace_bytes(100, 4, 4, ctypes.byref(o)) > 100 * 4 * 4
    assert L.tsqr_host_workspace_bytes(3, 4, 4, ctypes.byref(o)) == 0


def test_implicit_q_and_accuracy_check_argument_checks_need_no_gpu(tg):
    """tsqr_*_factor / tsqr_*_apply_qt / tsqr_*_form_q / tsqr_check reject
    bad sizes, leading dimensions, options and workspaces before any CUDA
    call, and their workspace queries answer on the CPU."""
    L = tg.lib()
    fake = ctypes.c_void_p(0x1000)
    o = tg._opts("plain")
    # factor: the tsqr_*_ex checks, plain precision only
    assert L.tsqr_s_factor(100, 8, fake, 99, fake, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    assert L.tsqr_s_factor(3, 8, fake, 3, fake, 8, fake, 1 << 20, ctypes.byref(o), None) == 1
    assert L.tsqr_s_factor(100, 8, fake, 100, fake, 8, fake, 1 << 20, ctypes.byref(tg._opts("tf32x3")), None) == 2
    assert L.tsqr_d_factor(100, 33, fake, 100, fake, 33, fake, 1 << 20, ctypes.byref(o), None) == 2
    assert L.tsqr_s_factor(1 << 20, 32, fake, 1 << 20, fake, 32, fake, 16, ctypes.byref(o), None) == 3
    # apply_qt
    args = lambda m, n, ldv, k, ldc, ldd, cwb: (m, n, fake, ldv, fake, 1 << 30, k, fake, ldc, fake, ldd, fake, cwb,
                                                None)
    assert L.tsqr_s_apply_qt(*args(100, 8, 99, 3, 100, 8, 1 << 20)) == 1   # ldv < m
    assert L.tsqr_s_apply_qt(*args(100, 8, 100, 0, 100, 8, 1 << 20)) == 1  # k < 1
    assert L.tsqr_s_apply_qt(*args(100, 8, 100, 3, 99, 8, 1 << 20)) == 1   # ldc < m
    assert L.tsqr_s_apply_qt(*args(100, 8, 100, 3, 100, 7, 1 << 20)) == 1  # ldd < n
    assert L.tsqr_s_apply_qt(*args(100, 65, 100, 3, 100, 65, 1 << 20)) == 2
    assert L.tsqr_d_apply_qt(*args(100, 33, 100, 3, 100, 33, 1 << 20)) == 2
    need = L.tsqr_apply_qt_workspace_bytes(1 << 20, 32, 5, 4)
    assert need > 0 and L.tsqr_apply_qt_workspace_bytes(100, 200, 5, 4) == 0
    assert L.tsqr_s_apply_qt(*args(1 << 20, 32, 1 << 20, 5, 1 << 20, 32, need - 1)) == 3
    # form_q
    assert L.tsqr_s_form_q(100, 8, fake, 99, fake, 1 << 20, None) == 1
    assert L.tsqr_d_form_q(100, 40, fake, 100, fake, 1 << 20, None) == 2
    # accuracy check
    res = tg.CheckResult()
    chk = lambda eb, m, n, lda, ldq, ldr, wb: L.tsqr_check(eb, m, n, fake, lda, fake, ldq, fake, ldr, 1e-4, 1e-5, fake,
                                                           wb, None, ctypes.byref(res))
    assert chk(4, 100, 8, 99, 100, 8, 1 << 20) == 1
    assert chk(4, 100, 8, 100, 99, 8, 1 << 20) == 1
    assert chk(4, 100, 8, 100, 100, 7, 1 << 20) == 1
    assert chk(3, 100, 8, 100, 100, 8, 1 << 20) == 1
    assert chk(8, 100, 8, 100, 100, 8, 16) == 3
    assert L.tsqr_check_workspace_bytes(1000, 32) >= 8 * 1000 * 32
    assert L.tsqr_check_workspace_bytes(0, 32) == 0


def test_qr_algorithm_option(tg):
    """The Householder algorithm of qr_*_ex: workspace query, panel limit,
    and an unknown algorithm rejected before any CUDA call."""
    L = tg.lib()
    fake = ctypes.c_void_p(0x1000)
    assert tg.qr_workspace_bytes(131072, 512, "float32", algorithm="householder") > 0
    assert tg.qr_workspace_bytes(131072, 512, "float32", algorithm="householder", panel=64) == 0
    o = tg._opts("plain")
    o.algorithm = 5
    assert L.qr_s_ex(1000, 64, fake, 1000, fake, 64, fake, 1 << 30, ctypes.byref(o), None) == 1
    o = tg._opts("plain", algorithm="householder", panel=64)
    assert L.qr_s_ex(1000, 64, fake, 1000, fake, 64, fake, 1 << 30, ctypes.byref(o), None) == 2
    o = tg._opts("plain", algorithm="householder")
    assert L.qr_s_ex(1000, 64, fake, 1000, fake, 64, fake, 16, ctypes.byref(o), None) == 3


def test_batched_tuning_table_needs_no_gpu(tg):
    """The autotuner's table: defaults, candidate tile heights, and argument
    checks of the tuning and setting calls (no CUDA call)."""
    L = tg.lib()
    assert [L.tsqr_batched_candidate_rows(c, 0) for c in range(4)] == [1024, 512, 512, 512]
    assert [L.tsqr_batched_candidate_rows(c, 1) for c in range(4)] == [512, 256, 256, 256]
    assert L.tsqr_batched_candidate_rows(4, 0) == -1 and L.tsqr_batched_candidate_rows(0, 2) == -1
    assert all(L.tsqr_batched_choice(c, b) == 0 for c in range(4) for b in range(3))
    assert L.tsqr_batched_choice(0, 3) == -1
    assert L.tsqr_batched_set_choice(2, 1, 1) == 0 and L.tsqr_batched_choice(2, 1) == 1
    assert L.tsqr_batched_set_choice(2, 1, 0) == 0
    assert L.tsqr_batched_set_choice(2, 1, 2) == 1 and L.tsqr_batched_set_choice(-1, 0, 0) == 1
    i64 = ctypes.c_int64 * 2
    assert L.tsqr_batched_tune_s(0, i64(100, 100), i64(8, 8), 3, None) == 1
    assert L.tsqr_batched_tune_s(2, i64(100, 100), i64(8, 65), 3, None) == 1
    assert L.tsqr_batched_tune_s(2, i64(100, 5), i64(8, 8), 3, None) == 1
    assert L.tsqr_batched_tune_s(2, i64(100, 100), i64(8, 8), 0, None) == 1


def test_noalloc_rejects_bad_arguments_before_any_cuda_call(tg):
    """tsqr_s_noalloc checks its arguments first, like the other entry points:
    n > 64 is unsupported; null matrices, short leading dimensions and m < n
    are invalid.  Nothing is launched, so fake pointers are enough."""
    fn = tg.lib().tsqr_s_noalloc
    fake = ctypes.c_void_p(0x1000)
    assert fn(1000, 65, fake, 1000, fake, 65, None) == 2   # TSQR_ERR_UNSUPPORTED
    assert fn(1000, 32, None, 1000, fake, 32, None) == 1   # A null
    assert fn(1000, 32, fake, 1000, None, 32, None) == 1   # R null
    assert fn(1000, 32, fake, 999, fake, 32, None) == 1    # lda < m
    assert fn(1000, 32, fake, 1000, fake, 31, None) == 1   # ldr < n
    assert fn(16, 32, fake, 16, fake, 32, None) == 1       # m < n
    assert fn(0, 32, fake, 1, fake, 32, None) == 1         # empty


def test_precision_form_options_and_reorth_sizes_need_no_gpu(tg):
    """fp64_scalars / fp64_root belong to the TF32X3 form of tsqr_*_ex
    (fp64_root for n <= 32); reorth adds an n x n factor to the workspace;
    option values other than 0 and 1 are invalid; the host, implicit-Q and
    blocked-QR entry points refuse the TSQR-only options before any CUDA
    call."""
    L = tg.lib()
    fake = ctypes.c_void_p(0x1000)
    o = tg._opts("plain")
    base = L.tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(o))
    o = tg._opts("plain", reorth=True)
    assert L.tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(o)) >= base + 32 * 32 * 4
    assert L.tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(tg._opts("plain", fp64_scalars=True))) == 0
    assert L.tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(tg._opts("tf32x3", fp64_scalars=True))) > 0
    assert L.tsqr_workspace_bytes(1 << 20, 32, 4, ctypes.byref(tg._opts("tf32x3", fp64_root=True))) > 0
    assert L.tsqr_workspace_bytes(1 << 20, 48, 4, ctypes.byref(tg._opts("tf32x3", fp64_root=True))) == 0
    bad = tg._opts("tf32x3")
    bad.fp64_scalars = 2
    assert L.tsqr_s_ex(1000, 32, fake, 1000, fake, 32, fake, 1 << 20, ctypes.byref(bad), None) == 1
    o = tg._opts("plain", fp64_root=True)
    assert L.tsqr_s_ex(1000, 32, fake, 1000, fake, 32, fake, 1 << 20, ctypes.byref(o), None) == 2
    o = tg._opts("plain", reorth=True)
    assert L.tsqr_s_ex(1 << 20, 32, fake, 1 << 20, fake, 32, fake, base, ctypes.byref(o), None) == 3
    assert L.tsqr_s_host(1000, 32, fake, 1000, fake, 1000, fake, 32, fake, 1 << 20, ctypes.byref(o), None) == 2
    assert L.tsqr_s_factor(1000, 32, fake, 1000, fake, 32, fake, 1 << 20, ctypes.byref(o), None) == 2
    o = tg._opts("tf32x3", fp64_scalars=True)
    assert L.qr_s_ex(1000, 64, fake, 1000, fake, 64, fake, 1 << 20, ctypes.byref(o), None) == 2
