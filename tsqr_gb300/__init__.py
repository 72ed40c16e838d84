"""tsqr_gb300 -- tall-skinny QR for one GB300 GPU (sm_103a).

Host-side mirror of the reference interface over the C ABI of
``libtsqr_gb300.so`` (declared in include/tsqr_gb300.h):

* ``tsqr(m, n, A, lda, R, ldr, d_work, ldwork, dtype)`` and
  ``qr(...)``: the reference signatures (TallShinnyQR.h:86-87,
  block_QR.h:72-73) on raw device pointers, legacy default stream;
* ``tsqr_(A, ...)`` / ``qr_(...)``: the same on torch CUDA tensors holding
  column-major matrices (shape (m, n), stride (1, lda)), on the current
  stream, with the precision form selectable;
* ``tsqr_batched_(As, ...)``: many uneven problems in one launch.

There is no CPU fallback: if the shared library is missing or was built for
another machine, importing the package raises.
"""
import ctypes
import os

__all__ = [
    "TsqrError", "PLAIN", "TF32X3", "BF16X3", "lib", "library_path", "tsqr", "qr", "tsqr_", "qr_",
    "tsqr_batched_", "batched_tune_", "batched_table", "profile_", "check_", "factor_", "apply_qt_", "form_q_", "Factorization", "workspace_bytes",
    "qr_workspace_bytes", "empty_colmajor", "to_colmajor",
]

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "libtsqr_gb300.so")

PLAIN, TF32X3, BF16X3 = 0, 1, 2
_PREC = {"plain": PLAIN, "tf32x3": TF32X3, "bf16x3": BF16X3, PLAIN: PLAIN, TF32X3: TF32X3, BF16X3: BF16X3}

STATUS = {0: "TSQR_OK", 1: "TSQR_ERR_INVALID_ARG", 2: "TSQR_ERR_UNSUPPORTED", 3: "TSQR_ERR_WORKSPACE",
          4: "TSQR_ERR_CUDA", 5: "TSQR_ERR_NO_DEVICE"}


class TsqrError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__("%s: %s (%s)" % (where, STATUS.get(status, status), _status_text(status)))


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("reorth", ctypes.c_int), ("panel", ctypes.c_int),
                ("algorithm", ctypes.c_int), ("fp64_scalars", ctypes.c_int), ("fp64_root", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class CheckResult(ctypes.Structure):
    _fields_ = [("backward_fro", ctypes.c_double), ("orth_fro", ctypes.c_double),
                ("backward_2", ctypes.c_double), ("orth_2", ctypes.c_double),
                ("gate_failures", ctypes.c_int64), ("first_row", ctypes.c_int64), ("first_col", ctypes.c_int64),
                ("first_value", ctypes.c_double), ("first_ref", ctypes.c_double)]


_i64 = ctypes.c_int64
_p = ctypes.c_void_p
_L = None

# name -> (argtypes, restype); the full export list of include/tsqr_gb300.h
EXPORTS = {
    "tsqr_workspace_bytes": ([_i64, _i64, ctypes.c_int, ctypes.POINTER(Opts)], ctypes.c_size_t),
    "qr_workspace_bytes": ([_i64, _i64, ctypes.c_int, ctypes.POINTER(Opts)], ctypes.c_size_t),
    "tsqr_s_ex": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "tsqr_d_ex": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "qr_s_ex": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "qr_d_ex": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "tsqr_float": ([ctypes.c_int] * 2 + [_p, ctypes.c_int, _p, ctypes.c_int, _p, ctypes.c_int], ctypes.c_int),
    "tsqr_double": ([ctypes.c_int] * 2 + [_p, ctypes.c_int, _p, ctypes.c_int, _p, ctypes.c_int], ctypes.c_int),
    "qr_float": ([ctypes.c_int] * 2 + [_p, ctypes.c_int, _p, ctypes.c_int, _p, ctypes.c_int], ctypes.c_int),
    "qr_double": ([ctypes.c_int] * 2 + [_p, ctypes.c_int, _p, ctypes.c_int, _p, ctypes.c_int], ctypes.c_int),
    "tsqr_batched_workspace_bytes": ([ctypes.c_int, _p, _p], ctypes.c_size_t),
    "tsqr_batched_s": ([ctypes.c_int, _p, _p, _p, _p, _p, _p, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p],
                       ctypes.c_int),
    "tsqr_s_noalloc": ([_i64, _i64, _p, _i64, _p, _i64, _p], ctypes.c_int),
    "tsqr_batched_tune_s": ([ctypes.c_int, _p, _p, ctypes.c_int, _p], ctypes.c_int),
    "tsqr_batched_choice": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "tsqr_batched_candidate_rows": ([ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "tsqr_batched_set_choice": ([ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "tsqr_host_workspace_bytes": ([_i64, _i64, ctypes.c_int, ctypes.POINTER(Opts)], ctypes.c_size_t),
    "tsqr_workspace_check": ([_p], ctypes.c_int),
    "tsqr_s_host": ([_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p],
                    ctypes.c_int),
    "tsqr_d_host": ([_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p],
                    ctypes.c_int),
    "tsqr_profile": ([ctypes.c_int, ctypes.c_int, _i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t,
                      ctypes.POINTER(Opts), _p, _p, _p, ctypes.c_int, _p], ctypes.c_int),
    "tsqr_s_factor": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "tsqr_d_factor": ([_i64, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t, ctypes.POINTER(Opts), _p], ctypes.c_int),
    "tsqr_apply_qt_workspace_bytes": ([_i64, _i64, _i64, ctypes.c_int], ctypes.c_size_t),
    "tsqr_s_apply_qt": ([_i64, _i64, _p, _i64, _p, ctypes.c_size_t, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t,
                         _p], ctypes.c_int),
    "tsqr_d_apply_qt": ([_i64, _i64, _p, _i64, _p, ctypes.c_size_t, _i64, _p, _i64, _p, _i64, _p, ctypes.c_size_t,
                         _p], ctypes.c_int),
    "tsqr_s_form_q": ([_i64, _i64, _p, _i64, _p, ctypes.c_size_t, _p], ctypes.c_int),
    "tsqr_d_form_q": ([_i64, _i64, _p, _i64, _p, ctypes.c_size_t, _p], ctypes.c_int),
    "tsqr_check_workspace_bytes": ([_i64, _i64], ctypes.c_size_t),
    "tsqr_check": ([ctypes.c_int, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, ctypes.c_double, ctypes.c_double, _p,
                    ctypes.c_size_t, _p, ctypes.POINTER(CheckResult)], ctypes.c_int),
    "tsqr_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "tsqr_version": ([], ctypes.c_char_p),
    "tsqr_debug_set_wait_limit": ([ctypes.c_int], ctypes.c_int),
}


def library_path():
    return _LIB_PATH


def lib():
    """Load libtsqr_gb300.so (raises if it has not been built)."""
    global _L
    if _L is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError("libtsqr_gb300.so not built; run `python -c 'import __graft_entry__ as g; g.build()'`"
                              " or `python tsqr_gb300/build.py`")
        L = ctypes.CDLL(_LIB_PATH)
        for name, (args, res) in EXPORTS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _L = L
    return _L


def _status_text(st):
    try:
        return lib().tsqr_status_string(int(st)).decode()
    except Exception:  # pragma: no cover - library missing while formatting an error
        return "?"


def _check(st, where):
    if st != 0:
        raise TsqrError(st, where)


_ALGO = {"block_gs": 0, "householder": 1, 0: 0, 1: 1}


def _opts(precision="plain", reorth=False, panel=0, algorithm="block_gs", fp64_scalars=False, fp64_root=False):
    o = Opts()
    o.precision = _PREC[precision]
    o.reorth = 1 if reorth else 0
    o.panel = int(panel)
    o.algorithm = _ALGO[algorithm]
    o.fp64_scalars = 1 if fp64_scalars else 0
    o.fp64_root = 1 if fp64_root else 0
    return o


def _elem(dtype):
    import torch
    if dtype in (torch.float32, "float32", "float", 4):
        return 4
    if dtype in (torch.float64, "float64", "double", 8):
        return 8
    raise TsqrError(1, "dtype %s" % (dtype,))


def workspace_bytes(m, n, dtype, precision="plain", reorth=False, fp64_scalars=False, fp64_root=False):
    o = _opts(precision, reorth, fp64_scalars=fp64_scalars, fp64_root=fp64_root)
    return int(lib().tsqr_workspace_bytes(m, n, _elem(dtype), ctypes.byref(o)))


def qr_workspace_bytes(m, n, dtype, precision="plain", reorth=False, panel=0, algorithm="block_gs"):
    o = _opts(precision, reorth, panel, algorithm)
    return int(lib().qr_workspace_bytes(m, n, _elem(dtype), ctypes.byref(o)))


# ---------------------------------------------------------------------------
# Reference signatures on raw device pointers (TallShinnyQR.h:86-87,
# block_QR.h:72-73).  dtype "float" or "double".
# ---------------------------------------------------------------------------
def tsqr(m, n, A, lda, R, ldr, d_work, ldwork, dtype="float"):
    fn = lib().tsqr_float if _elem(dtype) == 4 else lib().tsqr_double
    _check(fn(m, n, A, lda, R, ldr, d_work, ldwork), "tsqr")


def qr(m, n, A, lda, R, ldr, d_work, ldwork, dtype="float"):
    fn = lib().qr_float if _elem(dtype) == 4 else lib().qr_double
    _check(fn(m, n, A, lda, R, ldr, d_work, ldwork), "qr")


# ---------------------------------------------------------------------------
# torch tensors
# ---------------------------------------------------------------------------
def empty_colmajor(m, n, dtype=None, device="cuda", ld=None):
    """An (m, n) column-major tensor view with leading dimension ld >= m."""
    import torch
    ld = m if ld is None else ld
    return torch.empty((n, ld), dtype=dtype or torch.float32, device=device).t()[:m]


def to_colmajor(x):
    """Column-major copy of a 2-D tensor (no copy if it already is one)."""
    if x.dim() == 2 and x.stride(0) == 1 and x.stride(1) >= max(1, x.shape[0]):
        return x
    return x.t().contiguous().t()


def _ld(x):
    m, n = x.shape
    if x.stride(0) != 1 or (n > 1 and x.stride(1) < m):
        raise TsqrError(1, "matrix must be column-major (stride (1, ld>=m))")
    return x.stride(1) if n > 1 else max(m, x.stride(1))


def _stream_handle(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _work(nbytes, work, device):
    import torch
    if work is not None:
        if work.numel() * work.element_size() < nbytes:
            raise TsqrError(3, "workspace")
        return work, work.numel() * work.element_size()
    return torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device), max(nbytes, 1)


class Factorization:
    """The implicit-Q form left by factor_: A holds level 0 of the
    compact-WY tree and `work` the upper levels (keep both unchanged while
    the factorisation is in use); R is the n x n factor."""

    def __init__(self, A, R, work):
        self.A, self.R, self.work = A, R, work

    @property
    def shape(self):
        return tuple(self.A.shape)


def factor_(A, R=None, work=None, stream=None):
    """Up-sweep only (tsqr_*_factor): returns a Factorization; A is
    overwritten by the tree, not by Q.  Plain precision."""
    m, n = A.shape
    lda = _ld(A)
    if R is None:
        R = empty_colmajor(n, n, A.dtype, A.device)
    nbytes = workspace_bytes(m, n, A.dtype)
    if nbytes == 0:
        raise TsqrError(2, "factor_")
    w, wb = _work(nbytes, work, A.device)
    fn = lib().tsqr_s_factor if A.element_size() == 4 else lib().tsqr_d_factor
    o = _opts("plain")
    _check(fn(m, n, A.data_ptr(), lda, R.data_ptr(), _ld(R), w.data_ptr(), wb, ctypes.byref(o),
              _stream_handle(stream)), "factor_")
    return Factorization(A, R, w)


def apply_qt_(fac, C, D=None, work=None, stream=None):
    """D = Q^T C (n x k) for C (m x k, column-major) from a Factorization;
    C is only read."""
    A = fac.A
    m, n = A.shape
    k = C.shape[1]
    if C.shape[0] != m or C.dtype != A.dtype:
        raise TsqrError(1, "apply_qt_: C must be m x k of A's dtype")
    if D is None:
        D = empty_colmajor(n, k, A.dtype, A.device)
    nbytes = int(lib().tsqr_apply_qt_workspace_bytes(m, n, k, A.element_size()))
    if nbytes == 0:
        raise TsqrError(2, "apply_qt_")
    cw, cwb = _work(nbytes, work, A.device)
    fn = lib().tsqr_s_apply_qt if A.element_size() == 4 else lib().tsqr_d_apply_qt
    wb = fac.work.numel() * fac.work.element_size()
    _check(fn(m, n, A.data_ptr(), _ld(A), fac.work.data_ptr(), wb, k, C.data_ptr(), _ld(C), D.data_ptr(), _ld(D),
              cw.data_ptr(), cwb, _stream_handle(stream)), "apply_qt_")
    return D


def form_q_(fac, stream=None):
    """Down-sweep (tsqr_*_form_q): fac.A becomes the explicit thin Q."""
    A = fac.A
    m, n = A.shape
    fn = lib().tsqr_s_form_q if A.element_size() == 4 else lib().tsqr_d_form_q
    wb = fac.work.numel() * fac.work.element_size()
    _check(fn(m, n, A.data_ptr(), _ld(A), fac.work.data_ptr(), wb, _stream_handle(stream)), "form_q_")
    return A


def check_(A, Q, R, atol=1e-4, rtol=1e-5, work=None, stream=None):
    """Accuracy of Q R against the original A (column-major CUDA tensors of
    one dtype), computed on the GPU in FP64 by tsqr_check.  Returns a dict:
    backward_fro, orth_fro, backward_2, orth_2 (the reference's two printed
    figures), gate_failures and the first failing element (row, col, QR
    value, A value) of the all_close gate with tolerances atol / rtol."""
    m, n = Q.shape
    if A.shape != Q.shape or R.shape != (n, n) or A.dtype != Q.dtype or R.dtype != Q.dtype:
        raise TsqrError(1, "check_: shapes or dtypes disagree")
    nbytes = int(lib().tsqr_check_workspace_bytes(m, n))
    w, wb = _work(nbytes, work, Q.device)
    res = CheckResult()
    _check(lib().tsqr_check(Q.element_size(), m, n, A.data_ptr(), _ld(A), Q.data_ptr(), _ld(Q), R.data_ptr(), _ld(R),
                            float(atol), float(rtol), w.data_ptr(), wb, _stream_handle(stream), ctypes.byref(res)),
           "check_")
    out = {k: getattr(res, k) for k, _ in CheckResult._fields_}
    if out["gate_failures"] == 0:
        out["first_row"] = out["first_col"] = None
        out["first_value"] = out["first_ref"] = None
    return out


def tsqr_(A, R=None, precision="plain", work=None, stream=None, reorth=False, fp64_scalars=False, fp64_root=False):
    """Factor the column-major m x n CUDA tensor A in place: A <- Q.
    Returns R (n x n, column-major).  precision: "plain" or "tf32x3" (float32
    only).  reorth: one reorthogonalisation pass (a second TSQR of Q).
    fp64_scalars / fp64_root: options of the "tf32x3" form (FP64 Householder
    norm, beta and tau; FP64 root combine, n <= 32)."""
    import torch
    m, n = A.shape
    lda = _ld(A)
    if R is None:
        R = empty_colmajor(n, n, A.dtype, A.device)
    ldr = _ld(R)
    o = _opts(precision, reorth, fp64_scalars=fp64_scalars, fp64_root=fp64_root)
    nbytes = int(lib().tsqr_workspace_bytes(m, n, A.element_size(), ctypes.byref(o)))
    if nbytes == 0:
        raise TsqrError(2, "tsqr_ workspace (m=%d n=%d)" % (m, n))
    w, wb = _work(nbytes, work, A.device)
    fn = lib().tsqr_s_ex if A.dtype == torch.float32 else lib().tsqr_d_ex
    _check(fn(m, n, A.data_ptr(), lda, R.data_ptr(), ldr, w.data_ptr(), wb, ctypes.byref(o),
              _stream_handle(stream)), "tsqr_")
    return R


def tsqr_host_(A, Q=None, R=None, precision="plain", work=None, stream=None, device="cuda"):
    """TSQR of the column-major m x n host (CPU) tensor A, pinned for the
    copies to overlap: returns (Q, R) as host tensors (column-major).  The
    transfers are pipelined with the level-0 kernels on the device."""
    import torch
    m, n = A.shape
    lda = _ld(A)
    if Q is None:
        Q = torch.empty((n, m), dtype=A.dtype, pin_memory=A.is_pinned()).t()
    if R is None:
        R = torch.empty((n, n), dtype=A.dtype, pin_memory=A.is_pinned()).t()
    o = _opts(precision)
    nbytes = int(lib().tsqr_host_workspace_bytes(m, n, A.element_size(), ctypes.byref(o)))
    if nbytes == 0:
        raise TsqrError(2, "tsqr_host_ workspace (m=%d n=%d)" % (m, n))
    w, wb = _work(nbytes, work, torch.device(device))
    fn = lib().tsqr_s_host if A.dtype == torch.float32 else lib().tsqr_d_host
    _check(fn(m, n, A.data_ptr(), lda, Q.data_ptr(), _ld(Q), R.data_ptr(), _ld(R), w.data_ptr(), wb,
              ctypes.byref(o), _stream_handle(stream)), "tsqr_host_")
    return Q, R


def qr_(A, R=None, precision="plain", reorth=False, panel=0, work=None, stream=None, algorithm="block_gs"):
    """Blocked QR of the column-major CUDA tensor A in place (A <- Q).
    algorithm "block_gs": the reference's recursive block Gram-Schmidt;
    "householder": TSQR panels with reconstructed Householder vectors and
    compact-WY updates (orthogonal to working precision at any condition
    number)."""
    import torch
    m, n = A.shape
    lda = _ld(A)
    if R is None:
        R = empty_colmajor(n, n, A.dtype, A.device)
    ldr = _ld(R)
    o = _opts(precision, reorth, panel, algorithm)
    nbytes = int(lib().qr_workspace_bytes(m, n, A.element_size(), ctypes.byref(o)))
    if nbytes == 0:
        raise TsqrError(2, "qr_ workspace (m=%d n=%d)" % (m, n))
    w, wb = _work(nbytes, work, A.device)
    fn = lib().qr_s_ex if A.dtype == torch.float32 else lib().qr_d_ex
    _check(fn(m, n, A.data_ptr(), lda, R.data_ptr(), ldr, w.data_ptr(), wb, ctypes.byref(o),
              _stream_handle(stream)), "qr_")
    return R


def profile_(kind, A, R, precision="plain", reorth=False, panel=0, work=None, stream=None, max_launch=512,
             algorithm="block_gs"):
    """Run tsqr_ (kind "tsqr") or qr_ (kind "qr") with per-launch device
    timing.  Returns [(tag, ms), ...] in launch order; tag = kind*1000+level
    (1 factor, 2 apply, 3 gemm_tn, 4 reduce, 5 gemm_nn, 6 axpy, 7 tcgen05,
    8 batched, 9 apply_qt, 10 Householder reconstruction / small products /
    panel Q rows)."""
    m, n = A.shape
    o = _opts(precision, reorth, panel, algorithm)
    k = 0 if kind == "tsqr" else 1
    nbytes = (lib().tsqr_workspace_bytes if k == 0 else lib().qr_workspace_bytes)(m, n, A.element_size(),
                                                                                 ctypes.byref(o))
    w, wb = _work(int(nbytes), work, A.device)
    ms = (ctypes.c_float * max_launch)()
    tags = (ctypes.c_int * max_launch)()
    cnt = ctypes.c_int(0)
    _check(lib().tsqr_profile(k, A.element_size(), m, n, A.data_ptr(), _ld(A), R.data_ptr(), _ld(R), w.data_ptr(),
                              wb, ctypes.byref(o), _stream_handle(stream), ms, tags, max_launch,
                              ctypes.byref(cnt)), "profile_")
    return [(tags[i], ms[i]) for i in range(cnt.value)]


def batched_tune_(shapes, reps=3, stream=None):
    """Autotune the batched form for a list of (m, n) shapes: every candidate
    tile configuration of each (width class, height bucket) present is timed
    on synthetic matrices and the fastest kept (process-wide).  Returns the
    table: {(class, bucket): (candidate, tile rows)}."""
    count = len(shapes)
    i64 = ctypes.c_int64 * count
    m = i64(*[int(a) for a, _ in shapes])
    n = i64(*[int(b) for _, b in shapes])
    _check(lib().tsqr_batched_tune_s(count, m, n, int(reps), _stream_handle(stream)), "batched_tune_")
    return batched_table()


def batched_table():
    """The batched form's current choices: {(class, bucket): (candidate, rows)}."""
    L = lib()
    out = {}
    for c in range(4):
        for b in range(3):
            k = L.tsqr_batched_choice(c, b)
            out[(c, b)] = (k, L.tsqr_batched_candidate_rows(c, k))
    return out


def tsqr_batched_(As, Rs=None, precision="plain", work=None, stream=None):
    """Factor a list of column-major float32 CUDA tensors in one call: one
    launch per tree level and width class, no allocation and no host-to-device
    copy, so the call can be captured into a CUDA graph and replayed."""
    import torch
    count = len(As)
    if Rs is None:
        Rs = [empty_colmajor(a.shape[1], a.shape[1], a.dtype, a.device) for a in As]
    i64 = ctypes.c_int64 * count
    ptrs = ctypes.c_void_p * count
    m = i64(*[a.shape[0] for a in As])
    n = i64(*[a.shape[1] for a in As])
    lda = i64(*[_ld(a) for a in As])
    ldr = i64(*[_ld(r) for r in Rs])
    Ap = ptrs(*[a.data_ptr() for a in As])
    Rp = ptrs(*[r.data_ptr() for r in Rs])
    nbytes = int(lib().tsqr_batched_workspace_bytes(count, m, n))
    dev = As[0].device if count else torch.device("cuda")
    w, wb = _work(nbytes, work, dev)
    o = _opts(precision)
    _check(lib().tsqr_batched_s(count, Ap, m, n, lda, Rp, ldr, w.data_ptr(), wb, ctypes.byref(o),
                                _stream_handle(stream)), "tsqr_batched_")
    return Rs
