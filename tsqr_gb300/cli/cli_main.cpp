// cli_main.cpp -- the test_tsqr / test_qr command lines over libtsqr_gb300.
//
// Drop-in for the reference drivers test_tsqr.cu / test_qr.cu:
//   ./test_tsqr m n dtype      ./test_qr m n dtype      (dtype 1 = float, 2 = double)
// with the same defaults when fewer than three arguments are given
// (m = 13824, n = 32, double; test_tsqr.cu:112-128), the same input
// (std::default_random_engine(0) feeding uniform_real_distribution(-1, 1),
// column-major, lda = m; test_tsqr.cu:24-30), the same workspace the reference
// driver allocates (ldwork = 2*108*128 rows, ldwork*n elements;
// test_tsqr.cu:42-45), the same accuracy gate (QR vs A within abs 1e-4 /
// rel 1e-5, else "Error: tsqr" and exit(-1); utils.h:325-330), the same
// printed figures (|A-QR|/|A| and |I-Q^TQ|/n in spectral norm; utils.h:353)
// and the same timing protocol and line (warm-up then repeats, each
// re-uploading A outside the timed region; "tsqr Latency: x ms";
// test_tsqr.cu:62-90).  The accuracy check is the library's tsqr_check: the gate and
// both figures computed on the GPU in FP64 (Gram matrices, largest
// eigenvalue by Jacobi) instead of cuBLAS + cuSOLVER gesvd on a host copy.
// A final JSON line adds TFLOP/s and the Frobenius figures.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "tsqr_gb300.h"

#ifndef TSQR_CLI_QR
#define TSQR_CLI_QR 0
#endif

#if TSQR_CLI_QR
static const char* kName = "qr";
static const int kWarmup = 2, kRepeat = 5;  // test_qr.cu:13-14
#else
static const char* kName = "tsqr";
static const int kWarmup = 20, kRepeat = 50;  // test_tsqr.cu:13-14
#endif

#define CK(x)                                                                              \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            std::printf("CUDA error %d at %s:%d\n%s\n", (int)e_, __FILE__, __LINE__,      \
                        cudaGetErrorString(e_));                                           \
            std::exit(1);                                                                  \
        }                                                                                  \
    } while (0)

static tsqr_status call(float* A, float* R, float* W, int m, int n, int ldw) {
#if TSQR_CLI_QR
    return qr_float(m, n, A, m, R, n, W, ldw);
#else
    return tsqr_float(m, n, A, m, R, n, W, ldw);
#endif
}
static tsqr_status call(double* A, double* R, double* W, int m, int n, int ldw) {
#if TSQR_CLI_QR
    return qr_double(m, n, A, m, R, n, W, ldw);
#else
    return tsqr_double(m, n, A, m, R, n, W, ldw);
#endif
}

template <typename T>
static int run(int m, int n) {
    std::vector<T> A((size_t)m * n);
    std::default_random_engine eng(0U);
    std::uniform_real_distribution<T> dis(-1.0f, 1.0f);
    std::generate(A.begin(), A.end(), [&] { return dis(eng); });

    const int ldwork = 2 * 108 * 128;
    T *dA, *dA0, *dR, *dW;
    void* dC;
    const size_t check_bytes = tsqr_check_workspace_bytes(m, n);
    CK(cudaMalloc(&dA, sizeof(T) * A.size()));
    CK(cudaMalloc(&dA0, sizeof(T) * A.size()));
    CK(cudaMalloc(&dR, sizeof(T) * (size_t)n * n));
    CK(cudaMalloc(&dW, sizeof(T) * (size_t)ldwork * n));
    CK(cudaMalloc(&dC, check_bytes));
    CK(cudaMemcpy(dA, A.data(), sizeof(T) * A.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dA0, A.data(), sizeof(T) * A.size(), cudaMemcpyHostToDevice));
    tsqr_status st = call(dA, dR, dW, m, n, ldwork);
    if (st != TSQR_OK) {
        std::printf("%s: %s\n", kName, tsqr_status_string(st));
        return 1;
    }
    CK(cudaDeviceSynchronize());

    // Accuracy on the GPU in FP64: the QR vs A gate, then the spectral and
    // Frobenius figures.
    tsqr_check_result chk;
    st = tsqr_check((int)sizeof(T), m, n, dA0, m, dA, m, dR, n, 1e-4, 1e-5, dC, check_bytes, nullptr, &chk);
    if (st != TSQR_OK) {
        std::printf("check: %s\n", tsqr_status_string(st));
        return 1;
    }
    if (chk.gate_failures > 0) {
        std::printf("A[%lld, %lld] = %g A_ref[%lld, %lld] = %g Abs Diff: %g\n", (long long)chk.first_row,
                    (long long)chk.first_col, chk.first_value, (long long)chk.first_row, (long long)chk.first_col,
                    chk.first_ref, std::fabs(chk.first_value - chk.first_ref));
        std::printf("Error: %s\n", kName);
        std::exit(-1);
    }
    std::printf("|A-QR|/|A| = %.17f, |I-Q^TQ| / n = %.17f\n", chk.backward_2, chk.orth_2);

    cudaEvent_t start, stop;
    CK(cudaEventCreate(&start));
    CK(cudaEventCreate(&stop));
    float total = 0, t = 0;
    for (int i = 0; i < kWarmup; ++i) {
        CK(cudaMemcpy(dA, A.data(), sizeof(T) * A.size(), cudaMemcpyHostToDevice));
        CK(cudaDeviceSynchronize());
        call(dA, dR, dW, m, n, ldwork);
        CK(cudaDeviceSynchronize());
    }
    for (int i = 0; i < kRepeat; ++i) {
        CK(cudaMemcpy(dA, A.data(), sizeof(T) * A.size(), cudaMemcpyHostToDevice));
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(start, 0));
        call(dA, dR, dW, m, n, ldwork);
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(stop, 0));
        CK(cudaEventSynchronize(stop));
        CK(cudaEventElapsedTime(&t, start, stop));
        total += t;
    }
    total /= kRepeat;
    std::printf("%s Latency: %f ms\n", kName, total);
    const double F = 4.0 * m * (double)n * n - 4.0 / 3.0 * (double)n * n * n;
    std::printf("{\"cli\": \"%s\", \"m\": %d, \"n\": %d, \"dtype\": \"%s\", \"ms\": %.6f, \"tflops\": %.4f, "
                "\"backward_fro\": %.3e, \"orth_fro\": %.3e}\n",
                kName, m, n, sizeof(T) == 4 ? "float" : "double", total, F / (total * 1e-3) / 1e12,
                chk.backward_fro, chk.orth_fro);
    cudaFree(dA);
    cudaFree(dA0);
    cudaFree(dR);
    cudaFree(dW);
    cudaFree(dC);
    return 0;
}

int main(int argc, char* argv[]) {
    int m = 13824, n = 32, dtype = 2;  // test_tsqr.cu:113-114
    if (argc >= 4) {
        m = std::atoi(argv[1]);
        n = std::atoi(argv[2]);
        dtype = std::atoi(argv[3]);
    }
    if (dtype == 1) return run<float>(m, n);
    if (dtype == 2) return run<double>(m, n);
    return 0;
}
