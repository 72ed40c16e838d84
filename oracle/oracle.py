"""Python binding of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is test infrastructure: tests/, the smoke check and bench.py's CPU
baseline leg call it; the tsqr_gb300 product never does.  Matrices are numpy
arrays in Fortran (column-major) order, like the reference's buffers
(lda = m, test_tsqr.cu:30).

``ref_*`` functions restate the reference algorithm (see oracle.cpp for the
file:line each follows); ``householder_qr`` is the FP64 truth; ``metrics``
returns the backward error and orthogonality in FP64.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REFL = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


class OracleError(RuntimeError):
    pass


def lib():
    global _LIB
    if _LIB is None:
        from . import build_oracle
        path = build_oracle.build_oracle()
        L = ctypes.CDLL(path)
        for nm in ("orc_tile_qr_f", "orc_tile_qr_d"):
            getattr(L, nm).argtypes = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64]
            getattr(L, nm).restype = ctypes.c_int
        for nm in ("orc_ref_tsqr_f", "orc_ref_tsqr_d"):
            getattr(L, nm).argtypes = [_i64, _i64, _p, _i64, _p, _i64, _i64, _i64]
            getattr(L, nm).restype = ctypes.c_int
        for nm in ("orc_ref_qr_f", "orc_ref_qr_d"):
            getattr(L, nm).argtypes = [_i64, _i64, _p, _i64, _p, _i64, _i64, _i64, _i64]
            getattr(L, nm).restype = ctypes.c_int
        L.orc_householder_qr_d.argtypes = [_i64, _i64, _p, _i64, _p, _i64]
        L.orc_householder_qr_d.restype = ctypes.c_int
        for nm in ("orc_metrics_f", "orc_metrics_d"):
            getattr(L, nm).argtypes = [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p]
            getattr(L, nm).restype = None
        for nm in ("orc_sign_fix_f", "orc_sign_fix_d"):
            getattr(L, nm).argtypes = [_i64, _i64, _p, _i64, _p, _i64]
            getattr(L, nm).restype = None
        for nm in ("orc_fill_uniform_f", "orc_fill_uniform_d"):
            getattr(L, nm).argtypes = [_p, _i64, ctypes.c_uint]
            getattr(L, nm).restype = None
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_num_threads.argtypes = [ctypes.c_int]
        _LIB = L
    return _LIB


def _sfx(dtype):
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f"
    if dt == np.float64:
        return "d"
    raise OracleError("unsupported dtype %s" % dt)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _fortran(a, dtype=None):
    a = np.asarray(a, dtype=dtype)
    return np.asfortranarray(a)


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(t):
    lib().orc_set_num_threads(int(t))


def fill_uniform(m, n, dtype=np.float32, seed=0):
    """The reference's input (test_tsqr.cu:24-28): uniform[-1, 1) from
    std::default_random_engine(seed), generated in column-major order."""
    a = np.empty((m, n), dtype=dtype, order="F")
    getattr(lib(), "orc_fill_uniform_" + _sfx(dtype))(_ptr(a), m * n, seed)
    return a


def tile_qr(A):
    """Householder QR of one tile with explicit Q (kernelQR.h:69-291)."""
    A = _fortran(A)
    h, n = A.shape
    Q = np.empty_like(A, order="F")
    R = np.zeros((n, n), dtype=A.dtype, order="F")
    rc = getattr(lib(), "orc_tile_qr_" + _sfx(A.dtype))(h, n, _ptr(A), h, _ptr(Q), h, _ptr(R), n)
    if rc:
        raise OracleError("tile_qr rc=%d" % rc)
    return Q, R


def ref_tsqr(A, num_sm=108, block_size=128):
    """The reference TSQR schedule (TallShinnyQR.h:86-148) in A's precision.
    Returns (Q, R); raises OracleError on sizes the reference rejects."""
    Q = np.array(_fortran(A), order="F", copy=True)
    m, n = Q.shape
    R = np.zeros((n, n), dtype=Q.dtype, order="F")
    rc = getattr(lib(), "orc_ref_tsqr_" + _sfx(Q.dtype))(m, n, _ptr(Q), m, _ptr(R), n, num_sm, block_size)
    if rc:
        raise OracleError("ref_tsqr rc=%d (m=%d n=%d)" % (rc, m, n))
    return Q, R


def ref_qr(A, num_sm=108, block_size=128, nb=32):
    """The reference recursive blocked QR (block_QR.h:72-95)."""
    Q = np.array(_fortran(A), order="F", copy=True)
    m, n = Q.shape
    R = np.zeros((n, n), dtype=Q.dtype, order="F")
    rc = getattr(lib(), "orc_ref_qr_" + _sfx(Q.dtype))(m, n, _ptr(Q), m, _ptr(R), n, num_sm, block_size, nb)
    if rc:
        raise OracleError("ref_qr rc=%d (m=%d n=%d)" % (rc, m, n))
    return Q, R


def householder_qr(A):
    """FP64 Householder QR with explicit thin Q; diag(R) carries the
    reference's sign convention R_jj = -sign(x_j) ||x||."""
    Q = np.array(_fortran(A, np.float64), order="F", copy=True)
    m, n = Q.shape
    R = np.zeros((n, n), dtype=np.float64, order="F")
    rc = lib().orc_householder_qr_d(m, n, _ptr(Q), m, _ptr(R), n)
    if rc:
        raise OracleError("householder_qr rc=%d" % rc)
    return Q, R


def sign_fix(Q, R):
    """Normalise in place so diag(R) >= 0 (flip row i of R, column i of Q)."""
    assert Q.flags.f_contiguous and R.flags.f_contiguous and Q.dtype == R.dtype
    m, n = Q.shape
    getattr(lib(), "orc_sign_fix_" + _sfx(Q.dtype))(m, n, _ptr(Q), Q.shape[0], _ptr(R), R.shape[0])
    return Q, R


def metrics(A0, Q, R):
    """FP64 error figures of a factorisation A0 ~ Q R.

    backward:    ||A0 - QR||_F / ||A0||_F
    orth:        ||Q^T Q - I||_F
    backward_2:  ||A0 - QR||_2 / ||A0||_2      (the reference's printed figure, utils.h:353)
    orth_2_n:    ||I - Q^T Q||_2 / n           (the reference's printed figure, utils.h:353)
    """
    dt = np.result_type(A0.dtype, Q.dtype, R.dtype)
    if dt not in (np.float32, np.float64):
        dt = np.float64
    A0 = _fortran(A0, dt)
    Q = _fortran(Q, dt)
    R = _fortran(R, dt)
    m, n = Q.shape
    out = np.zeros(4, dtype=np.float64)
    getattr(lib(), "orc_metrics_" + _sfx(dt))(m, n, _ptr(A0), m, _ptr(Q), m, _ptr(R), n, _ptr(out))
    return {"backward": float(out[0]), "orth": float(out[1]),
            "backward_2": float(out[2]), "orth_2_n": float(out[3])}


def unit_roundoff(dtype):
    return 2.0 ** -24 if np.dtype(dtype) == np.float32 else 2.0 ** -53


# ---------------------------------------------------------------------------
# The reference's own kernels (oracle/_ref/ref_kernels.cubin), launched on a
# GPU by oracle/ref_launch.cpp.  Only for golden-vector generation and the
# reference-side timing; needs a CUDA device.
# ---------------------------------------------------------------------------
REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
REF_LDWORK = 2 * 108 * 128


def ref_cuda_available():
    return os.path.exists(REF_CUBIN)


def refl():
    global _REFL
    if _REFL is None:
        from . import build_oracle
        L = ctypes.CDLL(build_oracle.build_ref_launcher())
        L.refl_init.argtypes = [ctypes.c_char_p]
        L.refl_init.restype = ctypes.c_int
        ci = ctypes.c_int
        for nm in ("refl_tsqr_f", "refl_tsqr_d", "refl_qr_f", "refl_qr_d"):
            getattr(L, nm).argtypes = [ci, ci, _p, ci, _p, ci, _p, ci, _p]
            getattr(L, nm).restype = ci
        rc = L.refl_init(REF_CUBIN.encode())
        if rc:
            raise OracleError("refl_init rc=%d (cubin %s)" % (rc, REF_CUBIN))
        _REFL = L
    return _REFL


def ref_cuda_call(kind, A_dev, R_dev, work_dev, stream=0):
    """Run the reference tsqr/qr (kind 'tsqr' or 'qr') on torch CUDA tensors.

    A_dev is an (n, m) row-major tensor, i.e. the column-major m x n matrix
    (lda = m); R_dev is (n, n) the same way; work_dev has REF_LDWORK*n
    elements.  Returns the launcher's status (0 = launched)."""
    import torch
    assert A_dev.is_cuda and A_dev.is_contiguous()
    n, m = A_dev.shape
    sfx = "f" if A_dev.dtype == torch.float32 else "d"
    fn = getattr(refl(), "refl_%s_%s" % (kind, sfx))
    return fn(m, n, A_dev.data_ptr(), m, R_dev.data_ptr(), n, work_dev.data_ptr(), REF_LDWORK,
              ctypes.c_void_p(stream))
