// check.cu -- accuracy of a thin QR on the GPU (tsqr_check).
//
// Replaces the reference's host-driven accuracy check check_QR_accuracy
// (utils.h:317-455): there QR = Q R is formed by cuBLAS, copied to the host
// and compared element by element (all_close, utils.h:148-174, atol 1e-4 /
// rtol 1e-5), and the two printed figures ||A - QR||_2 / ||A||_2 and
// ||I - Q^T Q||_2 / n come from cuSOLVER gesvd, whose int-sized workspace
// breaks past m = 46,340.  Here everything stays on the device and in FP64:
//   * residual_kernel: E = A - Q R (a tiled FP64 product) and the same
//     element gate |(QR)_ij - A_ij| <= max(atol, rtol |A_ij|) (NaN fails),
//     counting failures and keeping the first one in the reference's
//     column-major traversal order (smallest i + j*m);
//   * gram_partial_kernel / gram_reduce_kernel: the n x n Gram matrices
//     E^T E, A^T A and Q^T Q as split-K partials over fixed row chunks,
//     summed in a fixed order (deterministic);
//   * the host derives the Frobenius figures from the traces and the
//     spectral ones from the largest eigenvalues of the n x n Grams
//     (cyclic Jacobi), since ||X||_2^2 = lambda_max(X^T X).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/tsqr_gb300.h"
#include "internal.h"

namespace tsqr {
namespace {

constexpr int kChunkRows = 4096;  // rows per split-K partial of a Gram matrix
constexpr int kTile = 32;         // Gram output tile and residual column block
constexpr int kResRows = 64;      // residual rows per CTA

struct CheckLayout {
    size_t E = 0, part = 0, gram = 0, ctr = 0, total = 0;
    int64_t chunks = 0;
};

CheckLayout check_layout(int64_t m, int64_t n) {
    CheckLayout L;
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    L.chunks = (m + kChunkRows - 1) / kChunkRows;
    L.E = 0;
    L.part = up(L.E + sizeof(double) * (size_t)m * (size_t)n);
    L.gram = up(L.part + sizeof(double) * (size_t)L.chunks * (size_t)n * (size_t)n);
    L.ctr = up(L.gram + 3 * sizeof(double) * (size_t)n * (size_t)n);
    L.total = up(L.ctr + 2 * sizeof(unsigned long long));
    return L;
}

// E = A - Q R for a kResRows x kTile block of E per CTA (256 threads, each
// 4 rows x 2 columns), the k loop staged through shared memory in FP64.
template <typename T>
__global__ void __launch_bounds__(256) residual_kernel(int64_t m, int n, const T* __restrict__ A, int64_t lda,
                                                       const T* __restrict__ Q, int64_t ldq,
                                                       const T* __restrict__ R, int64_t ldr, double* __restrict__ E,
                                                       double atol, double rtol, unsigned long long* fails,
                                                       unsigned long long* first) {
    __shared__ double Qs[kTile][kResRows + 1];  // Qs[k][row]
    __shared__ double Rs[kTile][kTile + 1];     // Rs[k][col]
    const int tid = threadIdx.x;
    const int tr = tid % 16, tc = tid / 16;  // rows tr + 16a, columns tc + 16b
    const int64_t row0 = (int64_t)blockIdx.x * kResRows;
    const int col0 = blockIdx.y * kTile;
    double acc[4][2] = {};
    for (int k0 = 0; k0 < n; k0 += kTile) {
        for (int e = tid; e < kTile * kResRows; e += 256) {
            const int r = e % kResRows, k = e / kResRows;
            const int64_t i = row0 + r;
            Qs[k][r] = (i < m && k0 + k < n) ? (double)Q[i + (int64_t)(k0 + k) * ldq] : 0.0;
        }
        for (int e = tid; e < kTile * kTile; e += 256) {
            const int k = e % kTile, c = e / kTile;
            Rs[k][c] = (k0 + k < n && col0 + c < n) ? (double)R[(k0 + k) + (int64_t)(col0 + c) * ldr] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < kTile; ++k) {
            double q[4], r[2];
#pragma unroll
            for (int a = 0; a < 4; ++a) q[a] = Qs[k][tr + 16 * a];
#pragma unroll
            for (int b = 0; b < 2; ++b) r[b] = Rs[k][tc + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b) acc[a][b] = fma(q[a], r[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            const int64_t i = row0 + tr + 16 * a;
            const int j = col0 + tc + 16 * b;
            if (i < m && j < n) {
                const double av = (double)A[i + (int64_t)j * lda];
                const double diff = acc[a][b] - av;
                E[i + (int64_t)j * m] = -diff;
                const double ad = fabs(diff);
                if (isnan(ad) || ad > fmax(atol, fabs(av) * rtol)) {
                    atomicAdd(fails, 1ull);
                    atomicMin(first, (unsigned long long)(i + (int64_t)j * m));
                }
            }
        }
}

// Tile pair (p, q), p <= q, of an n x n symmetric output with T = ceil(n/32)
// tiles per side, from its index in row-major order of the upper triangle.
__device__ __forceinline__ void tile_pair(int idx, int T, int& p, int& q) {
    p = 0;
    while (idx >= T - p) {
        idx -= T - p;
        ++p;
    }
    q = p + idx;
}

// Partial Gram matrix X_c^T X_c of row chunk c (blockIdx.y) for the 32 x 32
// output tile (p, q), p <= q (blockIdx.x), in FP64.  Each of the 256 threads
// keeps 4 outputs: column a = tid % 32 of tile p against columns
// b = tid / 32 + 8 s of tile q.  P[c] is n x n column-major; only tiles with
// p <= q are written.
template <typename TI>
__global__ void __launch_bounds__(256) gram_partial_kernel(int64_t m, int n, const TI* __restrict__ X, int64_t ldx,
                                                           double* __restrict__ P) {
    __shared__ double Xp[kTile][kTile + 1];  // [row][column of tile p]
    __shared__ double Xq[kTile][kTile + 1];  // [row][column of tile q]
    const int T = (n + kTile - 1) / kTile;
    int p, q;
    tile_pair(blockIdx.x, T, p, q);
    const int tid = threadIdx.x, a = tid % 32, b0 = tid / 32;
    const int cp = p * kTile, cq = q * kTile;
    const int64_t r0 = (int64_t)blockIdx.y * kChunkRows;
    const int64_t r1 = min(m, r0 + kChunkRows);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t rs = r0; rs < r1; rs += kTile) {
        for (int e = tid; e < kTile * kTile; e += 256) {
            const int r = e % kTile, c = e / kTile;
            const int64_t i = rs + r;
            const bool in = i < r1;
            Xp[r][c] = (in && cp + c < n) ? (double)X[i + (int64_t)(cp + c) * ldx] : 0.0;
            Xq[r][c] = (in && cq + c < n) ? (double)X[i + (int64_t)(cq + c) * ldx] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < kTile; ++r) {
            const double xa = Xp[r][a];
#pragma unroll
            for (int s = 0; s < 4; ++s) acc[s] = fma(xa, Xq[r][b0 + 8 * s], acc[s]);
        }
        __syncthreads();
    }
    double* Pc = P + (size_t)blockIdx.y * (size_t)n * (size_t)n;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int i = cp + a, j = cq + b0 + 8 * s;
        if (i < n && j < n) Pc[i + (size_t)j * n] = acc[s];
    }
}

// G = sum over chunks of P[c], in chunk order; the tiles below the diagonal
// are mirrored from the computed ones.
__global__ void gram_reduce_kernel(int n, int64_t chunks, const double* __restrict__ P, double* __restrict__ G) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= (int64_t)n * n) return;
    int i = (int)(o % n), j = (int)(o / n);
    if (i / kTile > j / kTile) {
        const int t = i;
        i = j;
        j = t;
    }
    const size_t src = (size_t)i + (size_t)j * n;
    double s = 0.0;
    for (int64_t c = 0; c < chunks; ++c) s += P[(size_t)c * (size_t)n * (size_t)n + src];
    G[o] = s;
}

template <typename TI>
cudaError_t gram(int64_t m, int n, const TI* X, int64_t ldx, double* P, int64_t chunks, double* G, cudaStream_t s) {
    const int T = (n + kTile - 1) / kTile;
    const dim3 grid((unsigned)(T * (T + 1) / 2), (unsigned)chunks);
    gram_partial_kernel<TI><<<grid, 256, 0, s>>>(m, n, X, ldx, P);
    const int64_t outs = (int64_t)n * n;
    gram_reduce_kernel<<<(unsigned)((outs + 255) / 256), 256, 0, s>>>(n, chunks, P, G);
    return cudaGetLastError();
}

// Eigenvalues of a symmetric n x n matrix (column-major) by cyclic Jacobi
// rotations; returns the diagonal after convergence (or 40 sweeps).
std::vector<double> sym_eigenvalues(std::vector<double> S, int n) {
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0, tot = 0;
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r) {
                const double v = S[r + (size_t)c * n] * S[r + (size_t)c * n];
                tot += v;
                if (r != c) off += v;
            }
        if (off == 0 || off <= 1e-30 * tot) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = S[p + (size_t)q * n];
                if (apq == 0) continue;
                const double th = (S[q + (size_t)q * n] - S[p + (size_t)p * n]) / (2 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double x = S[k + (size_t)p * n], y = S[k + (size_t)q * n];
                    S[k + (size_t)p * n] = c * x - s * y;
                    S[k + (size_t)q * n] = s * x + c * y;
                }
                for (int k = 0; k < n; ++k) {
                    const double x = S[p + (size_t)k * n], y = S[q + (size_t)k * n];
                    S[p + (size_t)k * n] = c * x - s * y;
                    S[q + (size_t)k * n] = s * x + c * y;
                }
            }
    }
    std::vector<double> d(n);
    for (int i = 0; i < n; ++i) d[i] = S[i + (size_t)i * n];
    return d;
}

template <typename T>
tsqr_status check_impl(int64_t m, int64_t n, const T* A, int64_t lda, const T* Q, int64_t ldq, const T* R,
                       int64_t ldr, double atol, double rtol, void* work, size_t work_bytes, cudaStream_t s,
                       tsqr_check_result* out) {
    if (!out || !A || !Q || !R || m < 1 || n < 1 || n > (1 << 16) || lda < m || ldq < m || ldr < n)
        return TSQR_ERR_INVALID_ARG;
    const CheckLayout L = check_layout(m, n);
    if (L.chunks > 65535) return TSQR_ERR_UNSUPPORTED;  // one grid row per chunk
    if (!work || work_bytes < L.total) return TSQR_ERR_WORKSPACE;
    char* base = static_cast<char*>(work);
    double* E = reinterpret_cast<double*>(base + L.E);
    double* P = reinterpret_cast<double*>(base + L.part);
    double* G = reinterpret_cast<double*>(base + L.gram);
    unsigned long long* ctr = reinterpret_cast<unsigned long long*>(base + L.ctr);
    const int ni = (int)n;
    const size_t nn = (size_t)n * (size_t)n;
    if (cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s) != cudaSuccess ||
        cudaMemsetAsync(ctr + 1, 0xff, sizeof(unsigned long long), s) != cudaSuccess)
        return TSQR_ERR_CUDA;
    const dim3 rgrid((unsigned)((m + kResRows - 1) / kResRows), (unsigned)((n + kTile - 1) / kTile));
    residual_kernel<T><<<rgrid, 256, 0, s>>>(m, ni, A, lda, Q, ldq, R, ldr, E, atol, rtol, ctr, ctr + 1);
    if (cudaGetLastError() != cudaSuccess) return TSQR_ERR_CUDA;
    if (gram<double>(m, ni, E, m, P, L.chunks, G, s) != cudaSuccess ||
        gram<T>(m, ni, A, lda, P, L.chunks, G + nn, s) != cudaSuccess ||
        gram<T>(m, ni, Q, ldq, P, L.chunks, G + 2 * nn, s) != cudaSuccess)
        return TSQR_ERR_CUDA;
    std::vector<double> g(3 * nn);
    unsigned long long c[2];
    if (cudaMemcpyAsync(g.data(), G, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(c, ctr, sizeof(c), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TSQR_ERR_CUDA;
    out->gate_failures = (int64_t)c[0];
    out->first_row = out->first_col = -1;
    out->first_value = out->first_ref = 0.0;
    if (c[0] > 0) {
        const int64_t idx = (int64_t)c[1];
        out->first_row = idx % m;
        out->first_col = idx / m;
        double e = 0;
        T a = 0;
        if (cudaMemcpy(&e, E + idx, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&a, A + out->first_row + out->first_col * lda, sizeof(T), cudaMemcpyDeviceToHost) !=
                cudaSuccess)
            return TSQR_ERR_CUDA;
        out->first_ref = (double)a;
        out->first_value = (double)a - e;  // (QR)_ij = A_ij - E_ij
    }
    const double* GE = g.data();
    const double* GA = g.data() + nn;
    std::vector<double> GQ(g.begin() + 2 * nn, g.end());
    double te = 0, ta = 0, fo = 0;
    for (int i = 0; i < ni; ++i) {
        te += GE[i + (size_t)i * n];
        ta += GA[i + (size_t)i * n];
        GQ[i + (size_t)i * n] -= 1.0;
    }
    for (double v : GQ) fo += v * v;
    out->backward_fro = ta > 0 ? std::sqrt(te / ta) : std::sqrt(te);
    out->orth_fro = std::sqrt(fo);
    double le = 0, la = 0, lo = 0;
    for (double v : sym_eigenvalues(std::vector<double>(GE, GE + nn), ni)) le = std::max(le, v);
    for (double v : sym_eigenvalues(std::vector<double>(GA, GA + nn), ni)) la = std::max(la, v);
    for (double v : sym_eigenvalues(GQ, ni)) lo = std::max(lo, std::fabs(v));
    out->backward_2 = la > 0 ? std::sqrt(le / la) : std::sqrt(le);
    out->orth_2 = lo / (double)n;
    return TSQR_OK;
}

}  // namespace
}  // namespace tsqr

extern "C" {

size_t tsqr_check_workspace_bytes(int64_t m, int64_t n) {
    if (m < 1 || n < 1) return 0;
    return tsqr::check_layout(m, n).total;
}

tsqr_status tsqr_check(int elem_bytes, int64_t m, int64_t n, const void* A, int64_t lda, const void* Q, int64_t ldq,
                       const void* R, int64_t ldr, double atol, double rtol, void* work, size_t work_bytes,
                       void* stream, tsqr_check_result* out) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (elem_bytes == 4)
        return tsqr::check_impl<float>(m, n, static_cast<const float*>(A), lda, static_cast<const float*>(Q), ldq,
                                       static_cast<const float*>(R), ldr, atol, rtol, work, work_bytes, s, out);
    if (elem_bytes == 8)
        return tsqr::check_impl<double>(m, n, static_cast<const double*>(A), lda, static_cast<const double*>(Q), ldq,
                                        static_cast<const double*>(R), ldr, atol, rtol, work, work_bytes, s, out);
    return TSQR_ERR_INVALID_ARG;
}

}  // extern "C"
