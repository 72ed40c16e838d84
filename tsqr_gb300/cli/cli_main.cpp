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
// test_tsqr.cu:62-90).  The checker is our own: spectral norms come from
// FP64 Gram matrices on the host (largest eigenvalue by Jacobi) instead of
// cuSOLVER gesvd.  A final JSON line adds TFLOP/s and the Frobenius figures.
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

// Largest eigenvalue of a symmetric n x n matrix (cyclic Jacobi).
static double lambda_max(std::vector<double> S, int n) {
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n * n; ++i) tot += S[i] * S[i];
        for (int p = 0; p < n; ++p)
            for (int q = 0; q < n; ++q)
                if (p != q) off += S[p + q * n] * S[p + q * n];
        if (off <= 1e-30 * tot || off == 0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = S[p + q * n];
                if (apq == 0) continue;
                double th = (S[q + q * n] - S[p + p * n]) / (2 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double a = S[k + p * n], b = S[k + q * n];
                    S[k + p * n] = c * a - s * b;
                    S[k + q * n] = s * a + c * b;
                }
                for (int k = 0; k < n; ++k) {
                    double a = S[p + k * n], b = S[q + k * n];
                    S[p + k * n] = c * a - s * b;
                    S[q + k * n] = s * a + c * b;
                }
            }
    }
    double mx = 0;
    for (int i = 0; i < n; ++i) mx = std::max(mx, S[i + i * n]);
    return mx;
}

template <typename T>
static int run(int m, int n) {
    std::vector<T> A((size_t)m * n), Q((size_t)m * n), R((size_t)n * n);
    std::default_random_engine eng(0U);
    std::uniform_real_distribution<T> dis(-1.0f, 1.0f);
    std::generate(A.begin(), A.end(), [&] { return dis(eng); });

    const int ldwork = 2 * 108 * 128;
    T *dA, *dR, *dW;
    CK(cudaMalloc(&dA, sizeof(T) * A.size()));
    CK(cudaMalloc(&dR, sizeof(T) * R.size()));
    CK(cudaMalloc(&dW, sizeof(T) * (size_t)ldwork * n));
    CK(cudaMemcpy(dA, A.data(), sizeof(T) * A.size(), cudaMemcpyHostToDevice));
    tsqr_status st = call(dA, dR, dW, m, n, ldwork);
    if (st != TSQR_OK) {
        std::printf("%s: %s\n", kName, tsqr_status_string(st));
        return 1;
    }
    CK(cudaDeviceSynchronize());
    CK(cudaMemcpy(Q.data(), dA, sizeof(T) * Q.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.data(), dR, sizeof(T) * R.size(), cudaMemcpyDeviceToHost));

    // Accuracy, in FP64: QR vs A gate, then spectral and Frobenius figures.
    std::vector<double> GE((size_t)n * n, 0.0), GA((size_t)n * n, 0.0), GQ((size_t)n * n, 0.0);
    std::vector<double> e(n), a(n), q(n);
    bool ok = true;
    for (int i = 0; i < m; ++i) {
        for (int c = 0; c < n; ++c) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += (double)Q[i + (size_t)k * m] * (double)R[k + (size_t)c * n];
            double av = (double)A[i + (size_t)c * m];
            double diff = std::fabs(s - av);
            if (ok && (std::isnan(diff) || diff > std::max(1e-4, std::fabs(av) * 1e-5))) {
                std::printf("A[%d, %d] = %g A_ref[%d, %d] = %g Abs Diff: %g\n", i, c, s, i, c, av, diff);
                ok = false;
            }
            e[c] = av - s;
            a[c] = av;
            q[c] = (double)Q[i + (size_t)c * m];
        }
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r) {
                GE[r + c * n] += e[r] * e[c];
                GA[r + c * n] += a[r] * a[c];
                GQ[r + c * n] += q[r] * q[c];
            }
    }
    if (!ok) {
        std::printf("Error: %s\n", kName);
        std::exit(-1);
    }
    double fe = 0, fa = 0, fo = 0;
    for (int i = 0; i < n; ++i) {
        fe += GE[i + i * n];
        fa += GA[i + i * n];
        GQ[i + i * n] -= 1.0;
    }
    for (double v : GQ) fo += v * v;
    std::vector<double> sq((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < n; ++r) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += GQ[r + k * n] * GQ[k + c * n];
            sq[r + c * n] = s;
        }
    const double back2 = std::sqrt(std::max(lambda_max(GE, n), 0.0) / lambda_max(GA, n));
    const double orth2 = std::sqrt(std::max(lambda_max(sq, n), 0.0)) / n;
    std::printf("|A-QR|/|A| = %.17f, |I-Q^TQ| / n = %.17f\n", back2, orth2);

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
                std::sqrt(fe / fa), std::sqrt(fo));
    cudaFree(dA);
    cudaFree(dR);
    cudaFree(dW);
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
