// block_QR.h -- drop-in replacement header for the reference's block_QR.h
// (dajunHuang/tsqr).
//
// Keeps the reference entry point (block_QR.h:72-73)
//     template <typename T>
//     void qr(int m, int n, T *A, int lda, T *R, int ldr, T *d_work, int ldwork);
// for T = float and double: recursive block Gram-Schmidt with TSQR panels
// (block_QR.h:75-94), A overwritten by Q, R written (including zeros in the
// lower-left blocks, which the reference leaves unwritten).  Forwards to
// libtsqr_gb300.  Any n is accepted (the reference needs n <= 32 or
// n / 2 a multiple of 32 at every level, block_QR.h:78-79).
#pragma once

#include <cstdio>

#include "TallShinnyQR.h"

#define N_B 32

template <typename T>
void qr(int m, int n, T *A, int lda, T *R, int ldr, T *d_work, int ldwork);

template <>
inline void qr<float>(int m, int n, float *A, int lda, float *R, int ldr, float *d_work, int ldwork) {
    tsqr_status s = qr_float(m, n, A, lda, R, ldr, d_work, ldwork);
    if (s != TSQR_OK) std::printf("qr: %s\n", tsqr_status_string(s));
}

template <>
inline void qr<double>(int m, int n, double *A, int lda, double *R, int ldr, double *d_work, int ldwork) {
    tsqr_status s = qr_double(m, n, A, lda, R, ldr, d_work, ldwork);
    if (s != TSQR_OK) std::printf("qr: %s\n", tsqr_status_string(s));
}
