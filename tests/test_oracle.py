"""CPU tests of the oracle itself: it is pinned before anything is checked
against it.

* The input stream is checked against an independent restatement of
  libstdc++'s minstd_rand0 + generate_canonical + uniform_real_distribution
  (the reference draws its inputs that way, test_tsqr.cu:24-28).
* The FP64 Householder QR is checked against LAPACK (scipy dgeqrf/dorgqr).
* The restated reference TSQR and blocked QR (FP32 and FP64) are checked for
  backward error and orthogonality, and against the FP64 truth.
* The reference's size rules (TallShinnyQR.h:92-109, block_QR.h:78-79) are
  enforced by the restatement.
Golden vectors produced by the reference's own CUDA kernels are checked in
test_golden.py.
"""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")


def minstd_uniform(count, dtype, seed=0):
    """libstdc++ std::default_random_engine(seed) (minstd_rand0: x <- 16807 x
    mod 2^31-1, seed 0 -> state 1) feeding uniform_real_distribution<T>(-1,1)
    through generate_canonical<T, digits>."""
    m = 2147483647
    x = 1 if seed % m == 0 else seed % m
    out = np.empty(count, dtype=dtype)
    if np.dtype(dtype) == np.float32:
        tmp = np.float32(2147483646.0)  # float(1 * r), r = max - min + 1
        for i in range(count):
            x = (16807 * x) % m
            s = np.float32(x - 1)
            r = s / tmp
            if r >= np.float32(1):
                r = np.nextafter(np.float32(1), np.float32(0))
            out[i] = r * np.float32(2) + np.float32(-1)
    else:
        r = 2147483646.0
        for i in range(count):
            x = (16807 * x) % m
            s = float(x - 1)
            x = (16807 * x) % m
            s = s + float(x - 1) * r
            t = r * r
            v = s / t
            if v >= 1.0:
                v = np.nextafter(1.0, 0.0)
            out[i] = v * 2.0 + -1.0
    return out


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_input_stream_matches_libstdcxx_restatement(orc, dtype):
    a = orc.fill_uniform(500, 2, dtype)
    ref = minstd_uniform(1000, dtype).reshape(2, 500).T  # column-major fill
    np.testing.assert_array_equal(a, ref)


def test_householder_fp64_matches_lapack(orc):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((3000, 40))
    Q, R = orc.householder_qr(A)
    Ql, Rl = scipy_linalg.qr(A, mode="economic")
    # Same reflector sign rule as LAPACK: diag(R) = -sign(a_jj) ||x||.
    np.testing.assert_allclose(R, Rl, rtol=0, atol=1e-12 * np.abs(Rl).max())
    np.testing.assert_allclose(Q, Ql, rtol=0, atol=1e-13)
    m = orc.metrics(A, Q, R)
    assert m["backward"] < 1e-14 and m["orth"] < 1e-13


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("m,n", [(27648, 32), (13824, 32), (4096, 16), (128, 32), (32, 32), (2048, 8), (27648 + 96, 32)])
def test_ref_tsqr_restatement(orc, dtype, m, n):
    A = orc.fill_uniform(m, n, dtype)
    Q, R = orc.ref_tsqr(A)
    u = orc.unit_roundoff(dtype)
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 10 * n * u
    assert met["orth"] <= 10 * n * u
    assert np.all(np.tril(R, -1) == 0)
    Qt, Rt = orc.householder_qr(A.astype(np.float64))
    Qs, Rs = Q.astype(np.float64, order="F"), R.astype(np.float64, order="F")
    orc.sign_fix(Qs, Rs)
    orc.sign_fix(Qt, Rt)
    assert np.abs(Rs - Rt).max() <= 100 * n * u * np.abs(Rt).max()
    assert np.abs(Qs - Qt).max() <= 100 * n * u


def test_ref_tsqr_size_rules(orc):
    A = orc.fill_uniform(1000, 24, np.float32)   # BLOCK_SIZE % n != 0 (TallShinnyQR.h:93)
    with pytest.raises(orc.OracleError):
        orc.ref_tsqr(A)
    A = orc.fill_uniform(130, 32, np.float32)    # (m % 128) % n != 0 (TallShinnyQR.h:129)
    with pytest.raises(orc.OracleError):
        orc.ref_tsqr(A)
    A = orc.fill_uniform(448, 64, np.float32)    # n > 32: 128 % 64 == 0 is allowed by :93 ...
    Q, R = orc.ref_tsqr(A)                       # ... the CPU restatement has no thread limit
    assert orc.metrics(A, Q, R)["backward"] < 1e-5


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ref_qr_restatement(orc, dtype):
    m, n = 27648, 128
    A = orc.fill_uniform(m, n, dtype)
    Q, R = orc.ref_qr(A)
    u = orc.unit_roundoff(dtype)
    met = orc.metrics(A, Q, R)
    assert met["backward"] <= 10 * n * u
    # classical Gram-Schmidt without reorthogonalisation: orthogonality is
    # kappa-dependent; random uniform inputs are well conditioned
    assert met["orth"] <= 100 * n * u
    with pytest.raises(orc.OracleError):
        orc.ref_qr(orc.fill_uniform(4096, 96, dtype))  # (n/2) % 32 != 0 (block_QR.h:79)


def test_tile_qr_convention(orc):
    """kernelQR.h:137-156: R_jj = -sign(x_j) ||x_j||, H = I - u u^T, ||u||^2 = 2."""
    A = np.asfortranarray(np.array([[3.0, 1.0], [4.0, 2.0], [0.0, 5.0]]))
    Q, R = orc.tile_qr(A)
    assert R[0, 0] == pytest.approx(-5.0)
    np.testing.assert_allclose(Q @ R, A, atol=1e-14)
    np.testing.assert_allclose(Q.T @ Q, np.eye(2), atol=1e-14)


def test_zero_column_gives_identity_reflector(orc):
    A = np.zeros((64, 4), order="F")
    A[:, 0] = 1.0
    Q, R = orc.tile_qr(A)
    assert np.all(np.isfinite(Q)) and np.all(np.isfinite(R))
    np.testing.assert_allclose(Q @ R, A, atol=1e-14)


def test_metrics_detect_a_planted_error(orc):
    A = orc.fill_uniform(2048, 16, np.float64)
    Q, R = orc.householder_qr(A)
    Q[5, 3] += 1e-3  # planted mistake, on the CPU
    met = orc.metrics(A, Q, R)
    assert met["backward"] > 1e-6 and met["orth"] > 1e-4
