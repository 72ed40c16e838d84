// TallShinnyQR.h -- drop-in replacement header for the reference's
// TallShinnyQR.h (dajunHuang/tsqr).
//
// Keeps the reference entry point (TallShinnyQR.h:86-87)
//     template <typename T>
//     void tsqr(int m, int n, T *A, int lda, T *R, int ldr, T *d_work, int ldwork);
// for T = float and double, with the same meaning: device pointers,
// column-major, A overwritten by the thin Q, R (n x n, ldr) written, launched
// on the legacy default stream and asynchronous.  It forwards to
// libtsqr_gb300 (link with -ltsqr_gb300).  Differences a caller can see:
//   * any n <= 64 (float) / 32 (double) and any m >= n are accepted (the
//     reference needs n <= 32, BLOCK_SIZE % n == 0, (m % 128) % n == 0 and
//     m <= (13824 / n) * 13824; TallShinnyQR.h:92-109, :129);
//   * a rejected call prints one line and returns, like the reference's
//     "not supported size" (TallShinnyQR.h:100-103), instead of asserting;
//   * d_work is used when it holds the library's workspace, otherwise the
//     library uses its own per-device buffer;
//   * no global state: concurrent calls on different devices are safe.
#pragma once

#include <cstdio>

#include "tsqr_gb300.h"

template <typename T>
void tsqr(int m, int n, T *A, int lda, T *R, int ldr, T *d_work, int ldwork);

template <>
inline void tsqr<float>(int m, int n, float *A, int lda, float *R, int ldr, float *d_work, int ldwork) {
    tsqr_status s = tsqr_float(m, n, A, lda, R, ldr, d_work, ldwork);
    if (s != TSQR_OK) std::printf("tsqr: %s\n", tsqr_status_string(s));
}

template <>
inline void tsqr<double>(int m, int n, double *A, int lda, double *R, int ldr, double *d_work, int ldwork) {
    tsqr_status s = tsqr_double(m, n, A, lda, R, ldr, d_work, ldwork);
    if (s != TSQR_OK) std::printf("tsqr: %s\n", tsqr_status_string(s));
}
