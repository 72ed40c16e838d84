// blocked_qr.cu -- recursive blocked QR over TSQR panels (plain precision).
//
// Replaces qr<T> (block_QR.h:72-95): recursive block classical Gram-Schmidt,
//   qr(A1);  R12 = A1^T A2;  A2 -= A1 R12;  qr(A2),
// with TSQR on panels of width <= panel (32, the reference's N_B,
// block_QR.h:5).  The reference's single naive kernel gemm_blockqr
// (block_QR.h:7-60: one thread per output, a length-m dot with stride-lda
// loads for op=T) becomes tiled SIMT kernels:
//   gemm_tn_fused (FP32): R12 = A1^T A2 in 32 x 32 output tiles, K = m split
//     across CTAs, the partial sums reduced in the same launch in a fixed
//     order (deterministic);
//   gemm_tn_partial + reduce_partials (FP64): the same product as split-K
//     partials of 64 x 64 tiles, then their sum;
//   gemm_nn: A2 = A2 - A1 R12, streamed over row blocks.
// Options the reference lacks: any split point (not only n/2 with
// (n/2) % 32 == 0, block_QR.h:78-79), a second projection (CGS2) when
// opts.reorth is set, and R21 written as zeros (the reference leaves it
// unwritten).
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace tsqr {

namespace {

constexpr int kTile = 64;  // output tile edge
constexpr int kKt = 16;    // k step through shared memory

// P_z (M x N, ld M) = sum over k in chunk z of A(k, i) * B(k, j);
// A is K x M, B is K x N, both column-major.
template <typename T>
__global__ void __launch_bounds__(256) gemm_tn_partial(int M, int N, int64_t K, const T* __restrict__ A,
                                                       int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                       T* __restrict__ P, int64_t kchunk) {
    pdl_begin();
    __shared__ T As[kKt][kTile + 1];
    __shared__ T Bs[kKt][kTile + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
    const int64_t kbeg = (int64_t)blockIdx.z * kchunk;
    const int64_t kend = min(K, kbeg + kchunk);
    T acc[4][4] = {};
    // the next k step's elements are loaded into registers while the current
    // one is multiplied out of shared memory
    T ra[4], rb[4];
    auto fetch = [&](int64_t k0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = tid + 256 * e;
            const int kk = idx % kKt, col = idx / kKt;
            const int64_t k = k0 + kk;
            ra[e] = (k < kend && i0 + col < M) ? A[k + (int64_t)(i0 + col) * lda] : T(0);
            rb[e] = (k < kend && j0 + col < N) ? B[k + (int64_t)(j0 + col) * ldb] : T(0);
        }
    };
    if (kbeg < kend) fetch(kbeg);
    for (int64_t k0 = kbeg; k0 < kend; k0 += kKt) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = tid + 256 * e;
            const int kk = idx % kKt, col = idx / kKt;
            As[kk][col] = ra[e];
            Bs[kk][col] = rb[e];
        }
        __syncthreads();
        if (k0 + kKt < kend) fetch(k0 + kKt);
#pragma unroll
        for (int kk = 0; kk < kKt; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][ty * 4 + u];
                b[u] = Bs[kk][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * b[v];
        }
        __syncthreads();
    }
    T* Pz = P + (int64_t)blockIdx.z * M * N;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty * 4 + u, j = j0 + tx * 4 + v;
            if (i < M && j < N) Pz[i + (int64_t)j * M] = acc[u][v];
        }
}

// C = alpha * sum_z P_z + beta * C  (C is M x N with ldc).  A CTA of 8
// warps takes 32 consecutive elements: warp w sums the partials z = w, w+8,
// ... of its lane's element (32 independent chains per warp, loads
// coalesced), then warp 0 adds the 8 warp sums in warp order, so the result
// is deterministic.
template <typename T>
__global__ void __launch_bounds__(256) reduce_partials(int M, int N, int nz, const T* __restrict__ P, T alpha,
                                                       T beta, T* C, int64_t ldc) {
    pdl_begin();
    __shared__ T s[8][32];
    const int64_t total = (int64_t)M * N;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t base = (int64_t)blockIdx.x * 32; base < total; base += (int64_t)gridDim.x * 32) {
        const int64_t e = base + lane;
        T a0 = T(0), a1 = T(0);
        if (e < total) {
            int z = w;
            for (; z + 8 < nz; z += 16) {
                a0 += P[(int64_t)z * total + e];
                a1 += P[(int64_t)(z + 8) * total + e];
            }
            if (z < nz) a0 += P[(int64_t)z * total + e];
        }
        s[w][lane] = a0 + a1;
        __syncthreads();
        if (w == 0 && e < total) {
            T t = s[0][lane];
#pragma unroll
            for (int q = 1; q < 8; ++q) t += s[q][lane];
            const int i = (int)(e % M), j = (int)(e / M);
            T* c = C + i + (int64_t)j * ldc;
            *c = (beta == T(0)) ? alpha * t : alpha * t + beta * *c;
        }
        __syncthreads();
    }
}
inline int reduce_blocks(int64_t total) { return (int)std::min<int64_t>(ceil_div(total, 32), 4096); }

// ---------------------------------------------------------------------------
// FP32 projection in one launch: C (n1 x n2, ldc) = alpha A^T B + beta C for
// A (K x n1) and B (K x n2), column-major.  The output is cut in 32 x 32
// tiles, so a 32-wide node computes no padding.  The K rows are split into S
// chunks per tile, one CTA each.  A CTA stages 64 rows of its 32 + 32
// columns per step in shared memory and reduces the step over four K slices
// of 64 threads (4 x 4 outputs per thread, 16-byte shared-memory reads).
// Its partial tile goes to global memory.  The last CTA of each group of g
// chunks to arrive (an atomic counter) sums the group's partials, and the
// last group sums the group partials into C.  Both sums run in a fixed order,
// so the result does not depend on which CTA arrives last.  No CTA waits on
// another; the last one resets the tile's counters for the next launch.
constexpr int kPT = 32;      // output tile edge
constexpr int kPRows = 64;   // rows staged per step
constexpr int kPCounters = 256 / sizeof(int);  // counter words start here in the workspace header
constexpr int kPHeader = 4096;                 // status word + counters
constexpr int kPMaxCounters = kPHeader / (int)sizeof(int) - kPCounters;

struct TnFusedPlan {
    int tiles_i = 1, ntiles = 1, S = 1, g = 1, G = 1;
    int64_t kchunk = 0;
    size_t part_bytes() const {  // chunk partials, then group partials
        return S > 1 ? (size_t)ntiles * (S + G) * kPT * kPT * sizeof(float) : 0;
    }
};

TnFusedPlan tn_fused_plan(int64_t n1, int64_t n2, int64_t K) {
    TnFusedPlan p;
    p.tiles_i = (int)ceil_div(n1, kPT);
    p.ntiles = p.tiles_i * (int)ceil_div(n2, kPT);
    // one wave of three CTAs per SM on GB300's 152 SMs (the register limit
    // of 256 threads at 75 registers), chunks of whole 64-row steps.  The
    // workspace query uses the same plan, so it takes the constant rather
    // than the device's count.
    const int64_t want = std::max<int64_t>(1, (3 * 152) / p.ntiles);
    p.kchunk = round_up(ceil_div(K, std::min<int64_t>(want, ceil_div(K, kPRows))), kPRows);
    p.S = (int)ceil_div(K, p.kchunk);
    p.g = 1;
    while ((int64_t)p.g * p.g < p.S) ++p.g;
    p.G = (int)ceil_div(p.S, p.g);
    if (p.S > 1 && (int64_t)p.ntiles * (p.G + 1) > kPMaxCounters) {  // too many counters: one chunk per tile
        p.S = 1;
        p.kchunk = round_up(std::max<int64_t>(K, 1), kPRows);
        p.g = p.G = 1;
    }
    return p;
}

struct TnFusedArgs {
    int n1, n2;
    int64_t K;
    const float* A;
    const float* B;
    int64_t ld;  // A and B share it
    float* C;
    int64_t ldc;
    float alpha, beta;
    int tiles_i, S, g, G;
    int64_t kchunk;
    float* part;  // [ntiles][S][1024]
    float* gpart;  // [ntiles][G][1024]
    int* cnt;      // [ntiles][G + 1], zero between launches
    int* err;      // status word (TMA form: a bounded wait gave up)
    int tries;     // polls of a bounded wait
};

// sum over z < n of q[z * 256] (float4 elements), in order of z, read from
// L2 (other CTAs wrote them): eight loads in flight per thread, the sum
// order unchanged (a missing term adds an exact zero)
__device__ __forceinline__ float4 sum_partials(const float4* q, int n) {
    constexpr int kStride = kPT * kPT / 4;
    float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int z0 = 0; z0 < n; z0 += 8) {
        float4 w[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
            w[e] = z0 + e < n ? __ldcg(q + (int64_t)(z0 + e) * kStride) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int e = 0; e < 8; ++e) u.x += w[e].x, u.y += w[e].y, u.z += w[e].z, u.w += w[e].w;
    }
    return u;
}

// The CTA's partial tile t (elements 4 tid .. 4 tid + 3 of the column-major
// 32 x 32 tile, in every thread) into C: directly when the tile has one
// chunk, else through the chunk partials and the two last-arriver sums.
__device__ __forceinline__ void tn_finish(const TnFusedArgs& p, float4 t, int tile, int chunk, int i0, int j0,
                                          int& s_last) {
    const int tid = threadIdx.x;
    auto store_c = [&](float4 s) {
        const float sv[4] = {s.x, s.y, s.z, s.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = 4 * tid + q, i = i0 + (e & 31), j = j0 + (e >> 5);
            if (i < p.n1 && j < p.n2) {
                float* c = p.C + i + (int64_t)j * p.ldc;
                *c = p.beta == 0.f ? p.alpha * sv[q] : p.alpha * sv[q] + p.beta * *c;
            }
        }
    };
    if (p.S == 1) {
        store_c(t);
        return;
    }
    constexpr int E = kPT * kPT;
    __stcg(reinterpret_cast<float4*>(p.part + ((int64_t)tile * p.S + chunk) * E) + tid, t);
    __threadfence();
    __syncthreads();
    int* cnt = p.cnt + tile * (p.G + 1);
    const int grp = chunk / p.g, g0 = grp * p.g, gn = min(p.g, p.S - g0);
    if (tid == 0) s_last = atomicAdd(cnt + grp, 1) == gn - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    float4 u = sum_partials(reinterpret_cast<const float4*>(p.part + ((int64_t)tile * p.S + g0) * E) + tid, gn);
    if (p.G > 1) {
        __stcg(reinterpret_cast<float4*>(p.gpart + ((int64_t)tile * p.G + grp) * E) + tid, u);
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(cnt + p.G, 1) == p.G - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        u = sum_partials(reinterpret_cast<const float4*>(p.gpart + (int64_t)tile * p.G * E) + tid, p.G);
    }
    store_c(u);
    if (tid <= p.G) cnt[tid] = 0;  // every CTA of the tile has counted: ready for the next launch
}

// TMA-fed form (A and B 16-byte aligned, lda a multiple of 4 floats): each
// 64-row step arrives as four 32 x 32 boxes (A rows 0-31 and 32-63, then B)
// with the 128-byte swizzle, in a ring of kPStages steps on mbarriers (the
// copies of the next three steps run under the current step's FMAs).
// Column c of a box holds 32 rows as 8 chunks of 16 bytes, chunk q at
// q ^ (c % 8).  Thread (ig, jg) of a K slice owns output rows ig + 8u and
// columns jg + 8v (u, v < 4): its eight 16-byte reads per 4 rows are free
// of bank conflicts.  Rows past the matrix end and columns past n1 / n2
// arrive as zeros; chunks are whole 64-row steps, so a CTA's last step never
// reaches into the next chunk.  The waits are bounded: after p.tries polls
// the CTA sets the status word, lets its copies in flight land and stops.
constexpr int kPStages = 4;
constexpr int kPBox = kPT * kPT * 4;                       // one 32 x 32 FP32 box
constexpr int kPStageBytes = 4 * kPBox;                    // A and B, 64 rows each
constexpr size_t kPTmaSmem = kPStages * kPStageBytes + 1024;  // + alignment of the swizzled boxes

__global__ void __launch_bounds__(256, 3)
    gemm_tn_tma(TnFusedArgs p, const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb) {
    pdl_begin();
    extern __shared__ unsigned char tn_raw[];
    __shared__ unsigned long long mbar[kPStages];
    __shared__ int s_last;
    unsigned char* base = tn_raw + ((1024 - (tc::smem_u32(tn_raw) & 1023)) & 1023);
    const uint32_t sbase = tc::smem_u32(base);
    const int tid = threadIdx.x;
    const int tile = blockIdx.x, chunk = blockIdx.y;
    const int i0 = (tile % p.tiles_i) * kPT, j0 = (tile / p.tiles_i) * kPT;
    const int64_t kbeg = (int64_t)chunk * p.kchunk;
    const int64_t kend = min(p.K, kbeg + p.kchunk);
    const int nst = (int)((kend - kbeg + kPRows - 1) / kPRows);
    if (tid == 0) {
        for (int b = 0; b < kPStages; ++b) tc::mbar_init(tc::smem_u32(&mbar[b]), 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int s) {  // thread 0
        const int b = s % kPStages;
        const uint32_t dst = sbase + b * kPStageBytes, mb = tc::smem_u32(&mbar[b]);
        const int x = (int)(kbeg + (int64_t)s * kPRows);
        tc::fence_smem_to_async();
        tc::mbar_arrive_expect_tx(mb, kPStageBytes);
        tc::tma_load_2d(dst, &ta, x, i0, mb);
        tc::tma_load_2d(dst + kPBox, &ta, x + 32, i0, mb);
        tc::tma_load_2d(dst + 2 * kPBox, &tb, x, j0, mb);
        tc::tma_load_2d(dst + 3 * kPBox, &tb, x + 32, j0, mb);
    };
    if (tid == 0)
        for (int s = 0; s < min(kPStages, nst); ++s) issue(s);

    const int sl = tid >> 6, lt = tid & 63, ig = lt & 7, jg = lt >> 3;
    float acc[4][4] = {};
    for (int s = 0; s < nst; ++s) {
        const int b = s % kPStages;
        const bool ok = tc::mbar_wait(tc::smem_u32(&mbar[b]), (uint32_t)(s / kPStages) & 1u, p.tries);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                if (p.err) atomicExch(p.err, 1);
                // the steps issued and not consumed: s .. s + kPStages - 1
                for (int q = s; q < min(s + kPStages, nst); ++q)
                    (void)tc::mbar_wait(tc::smem_u32(&mbar[q % kPStages]), (uint32_t)(q / kPStages) & 1u);
            }
            return;
        }
        // slice sl: rows 16 sl .. 16 sl + 15 of the step = box half sl / 2,
        // 4-row groups (sl % 2) * 4 .. + 3 of it
        const unsigned char* Ab = base + b * kPStageBytes + (sl >> 1) * kPBox;
        const unsigned char* Bb = Ab + 2 * kPBox;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int k4 = (sl & 1) * 4 + q;
            float4 a[4], bv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                a[u] = *reinterpret_cast<const float4*>(Ab + (ig + 8 * u) * 128 + ((k4 ^ ig) << 4));
#pragma unroll
            for (int v = 0; v < 4; ++v)
                bv[v] = *reinterpret_cast<const float4*>(Bb + (jg + 8 * v) * 128 + ((k4 ^ jg) << 4));
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    float c = acc[u][v];
                    c = fmaf(a[u].x, bv[v].x, c);
                    c = fmaf(a[u].y, bv[v].y, c);
                    c = fmaf(a[u].z, bv[v].z, c);
                    c = fmaf(a[u].w, bv[v].w, c);
                    acc[u][v] = c;
                }
        }
        __syncthreads();  // every thread is done with buffer b
        if (tid == 0 && s + kPStages < nst) issue(s + kPStages);
    }
    // the four slices' tiles (column-major, element j * 32 + i) in the ring's
    // first 16 KB: every copy has landed, all were waited for above
    float* red = reinterpret_cast<float*>(base);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) red[sl * kPT * kPT + (jg + 8 * v) * kPT + ig + 8 * u] = acc[u][v];
    __syncthreads();
    float4 t = *reinterpret_cast<const float4*>(red + 4 * tid);
#pragma unroll
    for (int q = 1; q < 4; ++q) {
        const float4 w = *reinterpret_cast<const float4*>(red + q * kPT * kPT + 4 * tid);
        t.x += w.x, t.y += w.y, t.z += w.z, t.w += w.w;
    }
    tn_finish(p, t, tile, chunk, i0, j0, s_last);
}

template <bool VEC>
__global__ void __launch_bounds__(256, 3) gemm_tn_fused(TnFusedArgs p) {
    pdl_begin();
    __shared__ __align__(16) float sm[2 * kPRows * kPT];  // A step | B step; later the four K slices' tiles
    __shared__ int s_last;
    float* As = sm;
    float* Bs = sm + kPRows * kPT;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tile = blockIdx.x, chunk = blockIdx.y;
    const int i0 = (tile % p.tiles_i) * kPT, j0 = (tile / p.tiles_i) * kPT;
    const int64_t kbeg = (int64_t)chunk * p.kchunk;
    const int64_t kend = min(p.K, kbeg + p.kchunk);

    // Loader: slot e of a thread covers rows 4kq..4kq+3 of one column gc of
    // the step (gc < 32: A's column i0 + gc, else B's column j0 + gc - 32);
    // a warp's slot is 4 columns x 32 rows, each column one 128-byte line.
    // Row r of column c is stored at [r][((c/4) ^ (r/4 % 8)) * 4 + c % 4]:
    // the stores of a warp hit 32 distinct banks, and a 16-byte read of 4
    // consecutive columns stays contiguous.
    const int kqa = lane & 7;
    const float* src[2];
    bool colok[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int gc = 4 * (warp * 2 + h) + (lane >> 3);
        const bool isA = gc < kPT;
        const int c = isA ? i0 + gc : j0 + gc - kPT;
        colok[h] = c < (isA ? p.n1 : p.n2);
        src[h] = (isA ? p.A : p.B) + (int64_t)(colok[h] ? c : 0) * p.ld;
    }
    float4 r[4];
    auto fetch = [&](int64_t k0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int64_t row = k0 + 4 * (8 * (e & 1) + kqa);
            const float* q = src[e >> 1] + row;
            if (!colok[e >> 1]) {
                r[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            } else if (VEC && row + 3 < kend) {
                r[e] = __ldg(reinterpret_cast<const float4*>(q));
            } else {
                r[e].x = row < kend ? __ldg(q) : 0.f;
                r[e].y = row + 1 < kend ? __ldg(q + 1) : 0.f;
                r[e].z = row + 2 < kend ? __ldg(q + 2) : 0.f;
                r[e].w = row + 3 < kend ? __ldg(q + 3) : 0.f;
            }
        }
    };

    // compute: slice sl takes rows 16 sl .. 16 sl + 15 of each step; thread
    // (ig, jg) of the slice owns rows 4ig.. and columns 4jg.. of the tile
    const int sl = tid >> 6, lt = tid & 63, ig = lt >> 3, jg = lt & 7;
    float acc[4][4] = {};
    if (kbeg < kend) fetch(kbeg);
    for (int64_t k0 = kbeg; k0 < kend; k0 += kPRows) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int kq = 8 * (e & 1) + kqa;
            const int gc = 4 * (warp * 2 + (e >> 1)) + (lane >> 3);
            float* dst = (gc < kPT ? As : Bs) + ((((gc & 31) >> 2) ^ (kq & 7)) << 2) + (gc & 3);
            dst[(4 * kq + 0) * kPT] = r[e].x;
            dst[(4 * kq + 1) * kPT] = r[e].y;
            dst[(4 * kq + 2) * kPT] = r[e].z;
            dst[(4 * kq + 3) * kPT] = r[e].w;
        }
        __syncthreads();
        if (k0 + kPRows < kend) fetch(k0 + kPRows);
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            const int k = 16 * sl + kk, s = (k >> 2) & 7;
            const float4 a = *reinterpret_cast<const float4*>(As + k * kPT + ((ig ^ s) << 2));
            const float4 b = *reinterpret_cast<const float4*>(Bs + k * kPT + ((jg ^ s) << 2));
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
        }
        __syncthreads();
    }

    // the four slices' tiles, column-major (element j*32 + i), summed in
    // slice order by the thread that owns elements 4t..4t+3
#pragma unroll
    for (int v = 0; v < 4; ++v)
        *reinterpret_cast<float4*>(sm + sl * kPT * kPT + (4 * jg + v) * kPT + 4 * ig) =
            make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
    __syncthreads();
    float4 t = *reinterpret_cast<const float4*>(sm + 4 * tid);
#pragma unroll
    for (int q = 1; q < 4; ++q) {
        const float4 w = *reinterpret_cast<const float4*>(sm + q * kPT * kPT + 4 * tid);
        t.x += w.x, t.y += w.y, t.z += w.z, t.w += w.w;
    }
    tn_finish(p, t, tile, chunk, i0, j0, s_last);
}

// ---------------------------------------------------------------------------
// FP32 update on CUDA cores: A2 (m x n2) += alpha A1 (m x n1) X (n1 x n2,
// ldx), A1 and A2 sharing lda, n1 <= 256.  A CTA owns a 32-column tile of
// A2 (blockIdx.y) and walks 128-row blocks (grid-stride, one wave).  X's
// n1 x 32 tile stays in shared memory for the whole launch.  A block's A1
// rows are staged 32 columns at a time (a straight copy of the column-major
// data, 16-byte stores); the next chunk, or the next block's first chunk
// and its A2 tile, are loaded into registers while the current chunk is
// multiplied.  Each thread owns 4 rows x 4 columns of the block and reads A1
// and X as 16-byte shared-memory vectors.
constexpr int kNR = 128;    // rows per block
constexpr int kNK = 32;     // K per staged chunk
constexpr int kNXs = 36;    // row stride of the X tile in shared memory (16-byte rows, 4-way store conflicts)
constexpr int kNMaxK = 256;

struct NnFusedArgs {
    int64_t m;
    int n1, n2;
    const float* A1;
    float* A2;
    int64_t lda;
    const float* X;
    int64_t ldx;
    float alpha;
};

size_t nn_fused_smem(int n1) { return ((size_t)round_up(n1, kNK) * kNXs + (size_t)kNK * kNR) * sizeof(float); }

template <bool VEC>
__global__ void __launch_bounds__(256, 2) gemm_nn_fused(NnFusedArgs p) {
    pdl_begin();
    extern __shared__ __align__(16) float nn_smem[];
    const int n1p = (p.n1 + kNK - 1) / kNK * kNK;
    float* Xs = nn_smem;              // [n1p][kNXs]
    float* As = nn_smem + n1p * kNXs;  // [kNK][kNR]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int j0 = blockIdx.y * 32;
    for (int e = tid; e < n1p * 32; e += 256) {
        const int i = e % n1p, j = e / n1p;
        Xs[i * kNXs + j] = (i < p.n1 && j0 + j < p.n2) ? p.X[i + (int64_t)(j0 + j) * p.ldx] : 0.f;
    }
    // compute: rows 4rg..4rg+3, columns 4cg..4cg+3 of the block
    const int rg = (warp & 3) * 8 + (lane & 7), cg = (warp >> 2) * 4 + (lane >> 3);
    const int64_t nblk = (p.m + kNR - 1) / kNR;

    // A1 chunk loader: float4 slot e = rows 4(idx%32).., column idx/32 of the chunk
    float4 ra[4];
    auto fetch_a = [&](int64_t row0, int kc) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = tid + 256 * e, kk = idx >> 5;
            const int64_t r = row0 + 4 * (idx & 31);
            const int k = kc + kk;
            const float* q = p.A1 + (int64_t)k * p.lda + r;
            if (k >= p.n1) {
                ra[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            } else if (VEC && r + 3 < p.m) {
                ra[e] = __ldg(reinterpret_cast<const float4*>(q));
            } else {
                ra[e].x = r < p.m ? __ldg(q) : 0.f;
                ra[e].y = r + 1 < p.m ? __ldg(q + 1) : 0.f;
                ra[e].z = r + 2 < p.m ? __ldg(q + 2) : 0.f;
                ra[e].w = r + 3 < p.m ? __ldg(q + 3) : 0.f;
            }
        }
    };
    // A2 tile of the thread: column 4cg + v, rows 4rg..4rg+3
    float4 rc[4];
    auto fetch_c = [&](int64_t row0) {
        const int64_t r = row0 + 4 * rg;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = j0 + 4 * cg + v;
            const float* q = p.A2 + (int64_t)(j < p.n2 ? j : 0) * p.lda + r;
            if (j >= p.n2) {
                rc[v] = make_float4(0.f, 0.f, 0.f, 0.f);
            } else if (VEC && r + 3 < p.m) {
                rc[v] = *reinterpret_cast<const float4*>(q);
            } else {
                rc[v].x = r < p.m ? q[0] : 0.f;
                rc[v].y = r + 1 < p.m ? q[1] : 0.f;
                rc[v].z = r + 2 < p.m ? q[2] : 0.f;
                rc[v].w = r + 3 < p.m ? q[3] : 0.f;
            }
        }
    };

    int64_t blk = blockIdx.x;
    if (blk < nblk) {
        fetch_a(blk * kNR, 0);
        fetch_c(blk * kNR);
    }
    for (; blk < nblk; blk += gridDim.x) {
        const int64_t row0 = blk * kNR;
        float4 c[4] = {rc[0], rc[1], rc[2], rc[3]};
        float acc[4][4] = {};
        for (int kc = 0; kc < p.n1; kc += kNK) {
            __syncthreads();  // the previous chunk's reads of As are done (and, first, Xs is written)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int idx = tid + 256 * e;
                *reinterpret_cast<float4*>(As + (idx >> 5) * kNR + 4 * (idx & 31)) = ra[e];
            }
            __syncthreads();
            if (kc + kNK < p.n1) {
                fetch_a(row0, kc + kNK);
            } else if (blk + gridDim.x < nblk) {
                fetch_a((blk + gridDim.x) * kNR, 0);
                fetch_c((blk + gridDim.x) * kNR);
            }
#pragma unroll 8
            for (int kk = 0; kk < kNK; ++kk) {
                const float4 a = *reinterpret_cast<const float4*>(As + kk * kNR + 4 * rg);
                const float4 x = *reinterpret_cast<const float4*>(Xs + (kc + kk) * kNXs + 4 * cg);
                const float av[4] = {a.x, a.y, a.z, a.w}, xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], xv[v], acc[u][v]);
            }
        }
        const int64_t r = row0 + 4 * rg;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int j = j0 + 4 * cg + v;
            if (j >= p.n2) continue;
            float4 o = c[v];
            o.x = fmaf(p.alpha, acc[0][v], o.x);
            o.y = fmaf(p.alpha, acc[1][v], o.y);
            o.z = fmaf(p.alpha, acc[2][v], o.z);
            o.w = fmaf(p.alpha, acc[3][v], o.w);
            float* q = p.A2 + (int64_t)j * p.lda + r;
            if (VEC && r + 3 < p.m) {
                *reinterpret_cast<float4*>(q) = o;
            } else {
                if (r < p.m) q[0] = o.x;
                if (r + 1 < p.m) q[1] = o.y;
                if (r + 2 < p.m) q[2] = o.z;
                if (r + 3 < p.m) q[3] = o.w;
            }
        }
    }
}

// C (M x N) = alpha * A (M x K) * B (K x N) + beta * C, column-major.
template <typename T>
__global__ void __launch_bounds__(256) gemm_nn(int64_t M, int N, int K, T alpha, const T* __restrict__ A,
                                               int64_t lda, const T* __restrict__ B, int64_t ldb, T beta, T* C,
                                               int64_t ldc) {
    pdl_begin();
    __shared__ T As[kKt][kTile + 1];
    __shared__ T Bs[kKt][kTile + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t i0 = (int64_t)blockIdx.x * kTile;
    const int j0 = blockIdx.y * kTile;
    T acc[4][4] = {};
    // the next k step's elements are loaded into registers while the current
    // one is multiplied out of shared memory
    T ra[4], rb[4];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = tid + 256 * e;
            {  // A tile: kKt columns of 64 contiguous rows
                const int row = idx % kTile, kk = idx / kTile;
                const int k = k0 + kk;
                ra[e] = (k < K && i0 + row < M) ? A[i0 + row + (int64_t)k * lda] : T(0);
            }
            {  // B tile: 64 columns of kKt contiguous k
                const int kk = idx % kKt, col = idx / kKt;
                const int k = k0 + kk;
                rb[e] = (k < K && j0 + col < N) ? B[k + (int64_t)(j0 + col) * ldb] : T(0);
            }
        }
    };
    if (K > 0) fetch(0);
    for (int k0 = 0; k0 < K; k0 += kKt) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int idx = tid + 256 * e;
            As[(idx / kTile)][idx % kTile] = ra[e];
            Bs[idx % kKt][idx / kKt] = rb[e];
        }
        __syncthreads();
        if (k0 + kKt < K) fetch(k0 + kKt);
#pragma unroll
        for (int kk = 0; kk < kKt; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][ty + 16 * u];
                b[u] = Bs[kk][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * b[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int64_t i = i0 + ty + 16 * u;
            const int j = j0 + tx * 4 + v;
            if (i < M && j < N) {
                T* c = C + i + (int64_t)j * ldc;
                *c = alpha * acc[u][v] + beta * *c;
            }
        }
}

template <typename T>
__global__ void axpy_block(int M, int N, const T* __restrict__ X, int64_t ldx, T* Y, int64_t ldy) {
    pdl_begin();
    const int64_t total = (int64_t)M * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % M), j = (int)(e / M);
        Y[i + (int64_t)j * ldy] += X[i + (int64_t)j * ldx];
    }
}

int panel_of(const tsqr_opts& o) { return o.panel > 0 ? o.panel : 32; }

int64_t split_of(int64_t n, int nb) {
    int64_t n1 = (n / 2) / nb * nb;
    return std::max<int64_t>(n1, nb);
}

struct GemmPlan {
    int nz;
    int64_t kchunk;
};

GemmPlan tn_plan(int64_t M, int64_t N, int64_t K) {
    const int64_t tiles = ceil_div(M, kTile) * ceil_div(N, kTile);
    int64_t nz = std::max<int64_t>(1, ceil_div(2 * 152, tiles));
    nz = std::min<int64_t>(nz, std::max<int64_t>(1, ceil_div(K, 256)));
    int64_t kchunk = round_up(ceil_div(K, nz), kKt);
    nz = ceil_div(K, kchunk);
    return {(int)nz, kchunk};
}

// Bytes of partial sums proj_tn needs for an n1 x n2 projection over K rows.
template <typename T>
size_t proj_tn_part_bytes(int64_t n1, int64_t n2, int64_t K) {
    if (std::is_same<T, float>::value) return tn_fused_plan(n1, n2, K).part_bytes();
    return (size_t)tn_plan(n1, n2, K).nz * n1 * n2 * sizeof(T);
}

// Workspace layout: [status word | tsqr region | partial sums | reorth temp].
// The precision form (FP32, TF32X3) sizes the TSQR region for the
// precision-form TSQR and the partial sums for the tcgen05 split-K GEMM.
struct QrWs {
    size_t err_bytes = kPHeader, tsqr_bytes = 0, part_bytes = 0, tmp_bytes = 0;
    size_t total() const { return err_bytes + tsqr_bytes + part_bytes + tmp_bytes; }
};

// The tensor-core forms (FP32 only): TF32X3, or BF16X3, whose GEMMs use
// BF16 hi/lo splits (the TSQR panels stay on the TF32x3 tensor-core form).
template <typename T>
bool use_tc(const tsqr_opts& o) {
    return sizeof(T) == 4 && (o.precision == TSQR_PRECISION_TF32X3 || o.precision == TSQR_PRECISION_BF16X3);
}
template <typename T>
bool use_bf16(const tsqr_opts& o) {
    return sizeof(T) == 4 && o.precision == TSQR_PRECISION_BF16X3;
}

// The projection R12 = A1^T A2 runs on the tensor cores only when both sides
// are at least 256 wide.  Measured at 131072 rows: 0.70 ms (tensor) vs
// 0.79 ms (SIMT) at 256x256, but 0.24 vs 0.205 ms at 128x128 and 0.09-0.16
// vs 0.055 ms below; the narrower products stay in FP32 on CUDA cores.
bool tc_projection(bool tc, int64_t n1, int64_t n2) { return tc && n1 >= 256 && n2 >= 256; }

template <typename T>
void qr_ws_walk(int64_t m, int64_t n, int nb, bool reorth, bool tc, QrWs* w) {
    if (n <= nb) {
        const size_t b = tc ? tsqr_precision_workspace(m, n) : tsqr_plain_workspace<T>(m, n);
        w->tsqr_bytes = std::max(w->tsqr_bytes, (size_t)round_up((int64_t)b, 256));
        return;
    }
    const int64_t n1 = split_of(n, nb), n2 = n - n1;
    const size_t pb = tc_projection(tc, n1, n2) ? (size_t)tc_tn_splits(n1, n2, m) * n1 * n2 * sizeof(T)
                                                : proj_tn_part_bytes<T>(n1, n2, m);
    w->part_bytes = std::max(w->part_bytes, (size_t)round_up((int64_t)pb, 256));
    if (reorth) w->tmp_bytes = std::max(w->tmp_bytes, (size_t)round_up(n1 * n2 * (int64_t)sizeof(T), 256));
    qr_ws_walk<T>(m, n1, nb, reorth, tc, w);
    qr_ws_walk<T>(m, n2, nb, reorth, tc, w);
}

// C (n1 x n2, ldc) = A1^T A2 (+ beta C) on the tensor cores (FP32 only).
template <typename T>
void proj_tn_tc(int64_t m, int64_t n1, int64_t n2, const T* A1, const T* A2, int64_t lda, T* P, T* C, int64_t ldc,
                T beta, int* err, cudaStream_t s, bool bf16) {
    if constexpr (std::is_same<T, float>::value) {
        const int nz = tc_gemm_tn((int)n1, (int)n2, m, A1, lda, A2, lda, P, err, s, bf16);
        log_launch(kTagTc + 100, s);
        launch_pdl(reduce_partials<T>, dim3(reduce_blocks(n1 * n2)), dim3(256), 0, s, (int)n1, (int)n2, nz,
                   (const T*)P, T(1), beta, C, ldc);
        log_launch(kTagReduce, s);
    }
}

// A2 (m x n2) -= A1 (m x n1) X (n1 x n2, ldx) in FP32 on CUDA cores
// (gemm_nn_fused, n1 <= 256).
void update_nn_fused(int64_t m, int64_t n1, int64_t n2, const float* A1, int64_t lda, const float* X, int64_t ldx,
                     float* A2, cudaStream_t s) {
    NnFusedArgs a;
    a.m = m;
    a.n1 = (int)n1;
    a.n2 = (int)n2;
    a.A1 = A1;
    a.A2 = A2;
    a.lda = lda;
    a.X = X;
    a.ldx = ldx;
    a.alpha = -1.f;
    const int tj = (int)ceil_div(n2, 32);
    const int64_t resident = 2 * (int64_t)device_sm_count();
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(m, kNR), ceil_div(resident, tj)));
    const size_t smem = nn_fused_smem((int)n1);
    static PerDeviceOnce attr;
    attr.run([] {
        const int mx = (int)nn_fused_smem(kNMaxK);
        cudaFuncSetAttribute(gemm_nn_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(gemm_nn_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    });
    const bool vec = lda % 4 == 0 && reinterpret_cast<uintptr_t>(A1) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(A2) % 16 == 0;
    if (vec)
        launch_pdl(gemm_nn_fused<true>, dim3((unsigned)gx, (unsigned)tj), dim3(256), smem, s, a);
    else
        launch_pdl(gemm_nn_fused<false>, dim3((unsigned)gx, (unsigned)tj), dim3(256), smem, s, a);
    log_launch(kTagGemmNN, s);
}

// The tensor-core forms' updates run on the tcgen05 GEMM only when the
// panel is wider than kNnTcMin.  Measured at 131,072 x 512 (TF32x3,
// reorthogonalised) with the register-staged tcgen05 kernel: 6.156 ms with
// the CUDA-core kernel up to 64 columns, 5.966 ms up to 128, 6.077 ms up
// to 256; with the TMA-fed one (tc_nn_tma_kernel, 256 threads): 4.531 ms
// up to 128, 4.386 ms up to 64.
constexpr int64_t kNnTcMin = 64;

// A2 (m x n2) -= A1 (m x n1) X (n1 x n2) in a tensor-core form (FP32 only).
template <typename T>
void update_nn_tc(int64_t m, int64_t n1, int64_t n2, const T* A1, int64_t lda, const T* X, int64_t ldx, T* A2,
                  int* err, cudaStream_t s, bool bf16) {
    if constexpr (std::is_same<T, float>::value) {
        if (n1 <= kNnTcMin) return update_nn_fused(m, n1, n2, A1, lda, X, ldx, A2, s);
        tc_gemm_nn(m, (int)n2, (int)n1, -1.f, A1, lda, X, ldx, A2, lda, err, s, bf16);
        log_launch(kTagTc + 101, s);
    }
}

// A2 (m x n2) -= A1 (m x n1) X (n1 x n2, ldx) on CUDA cores, plain form.
template <typename T>
void update_nn(int64_t m, int64_t n1, int64_t n2, const T* A1, int64_t lda, const T* X, int64_t ldx, T* A2,
               cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        if (n1 <= kNMaxK) return update_nn_fused(m, n1, n2, A1, lda, X, ldx, A2, s);
    }
    dim3 g((unsigned)ceil_div(m, kTile), (unsigned)ceil_div(n2, kTile));
    launch_pdl(gemm_nn<T>, g, dim3(256), 0, s, m, (int)n2, (int)n1, T(-1), A1, lda, X, ldx, T(1), A2, lda);
    log_launch(kTagGemmNN, s);
}

// C (n1 x n2, ldc) = A1^T A2 (+ beta C) on CUDA cores.  FP32: one launch of
// gemm_tn_fused (cnt: the workspace's counter words, zero between
// launches); FP64: split-K partials, then their sum.
template <typename T>
tsqr_status proj_tn(int64_t m, int64_t n1, int64_t n2, const T* A1, const T* A2, int64_t lda, T* P, T* C,
                    int64_t ldc, T beta, int* cnt, int* err, cudaStream_t s) {
    if constexpr (std::is_same<T, float>::value) {
        const TnFusedPlan fp = tn_fused_plan(n1, n2, m);
        TnFusedArgs a;
        a.n1 = (int)n1;
        a.n2 = (int)n2;
        a.K = m;
        a.A = A1;
        a.B = A2;
        a.ld = lda;
        a.C = C;
        a.ldc = ldc;
        a.alpha = 1.f;
        a.beta = beta;
        a.tiles_i = fp.tiles_i;
        a.S = fp.S;
        a.g = fp.g;
        a.G = fp.G;
        a.kchunk = fp.kchunk;
        a.part = P;
        a.gpart = P + (size_t)fp.ntiles * fp.S * kPT * kPT;
        a.cnt = cnt;
        a.err = err;
        a.tries = wait_tries().load(std::memory_order_relaxed);
        const dim3 g((unsigned)fp.ntiles, (unsigned)fp.S);
        CUtensorMap ta, tb;
        if (m + kPRows <= INT32_MAX && tensor_map_f32(&ta, A1, lda, m, n1, 32, 32, true) &&
            tensor_map_f32(&tb, A2, lda, m, n2, 32, 32, true)) {
            static PerDeviceOnce attr;
            attr.run([] {
                cudaFuncSetAttribute(gemm_tn_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPTmaSmem);
            });
            launch_pdl(gemm_tn_tma, g, dim3(256), kPTmaSmem, s, a, ta, tb);
            log_launch(kTagGemmTN, s);
            return TSQR_OK;
        }
        const bool vec = lda % 4 == 0 && reinterpret_cast<uintptr_t>(A1) % 16 == 0 &&
                         reinterpret_cast<uintptr_t>(A2) % 16 == 0;
        if (vec)
            launch_pdl(gemm_tn_fused<true>, g, dim3(256), 0, s, a);
        else
            launch_pdl(gemm_tn_fused<false>, g, dim3(256), 0, s, a);
        log_launch(kTagGemmTN, s);
        return TSQR_OK;
    }
    GemmPlan gp = tn_plan(n1, n2, m);
    dim3 g((unsigned)ceil_div(n1, kTile), (unsigned)ceil_div(n2, kTile), (unsigned)gp.nz);
    launch_pdl(gemm_tn_partial<T>, g, dim3(256), 0, s, (int)n1, (int)n2, m, A1, lda, A2, lda, P, gp.kchunk);
    log_launch(kTagGemmTN, s);
    launch_pdl(reduce_partials<T>, dim3(reduce_blocks(n1 * n2)), dim3(256), 0, s, (int)n1, (int)n2, gp.nz,
               (const T*)P, T(1), beta, C, ldc);
    log_launch(kTagReduce, s);
    return TSQR_OK;
}


template <typename T>
tsqr_status qr_rec(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, char* ws, const QrWs& w,
                   const tsqr_opts& o, cudaStream_t s) {
    const int nb = panel_of(o);
    const bool tc = use_tc<T>(o);
    char* tws = ws + w.err_bytes;
    if (n <= nb) {
        if constexpr (std::is_same<T, float>::value) {
            if (tc) return tsqr_precision(m, n, A, lda, R, ldr, tws, w.tsqr_bytes, s);
        }
        return tsqr_plain<T>(m, n, A, lda, R, ldr, tws, w.tsqr_bytes, s);
    }
    const int64_t n1 = split_of(n, nb), n2 = n - n1;
    T* A1 = A;
    T* A2 = A + n1 * lda;
    T* R11 = R;
    T* R12 = R + n1 * ldr;
    T* R22 = R + n1 * ldr + n1;
    int* err = reinterpret_cast<int*>(ws);
    int* cnt = err + kPCounters;
    T* P = reinterpret_cast<T*>(tws + w.tsqr_bytes);
    T* tmp = reinterpret_cast<T*>(tws + w.tsqr_bytes + w.part_bytes);
    tsqr_status st = qr_rec<T>(m, n1, A1, lda, R11, ldr, ws, w, o, s);
    if (st != TSQR_OK) return st;
    const bool tcp = tc_projection(tc, n1, n2);
    if (tc) {
        if (tcp)
            proj_tn_tc<T>(m, n1, n2, A1, A2, lda, P, R12, ldr, T(0), err, s, use_bf16<T>(o));
        else
            proj_tn<T>(m, n1, n2, A1, A2, lda, P, R12, ldr, T(0), cnt, err, s);
        update_nn_tc<T>(m, n1, n2, A1, lda, R12, ldr, A2, err, s, use_bf16<T>(o));
    } else {
        proj_tn<T>(m, n1, n2, A1, A2, lda, P, R12, ldr, T(0), cnt, err, s);
        update_nn<T>(m, n1, n2, A1, lda, R12, ldr, A2, s);
    }
    if (o.reorth) {
        if (tc) {
            if (tcp)
                proj_tn_tc<T>(m, n1, n2, A1, A2, lda, P, tmp, n1, T(0), err, s, use_bf16<T>(o));
            else
                proj_tn<T>(m, n1, n2, A1, A2, lda, P, tmp, n1, T(0), cnt, err, s);
            update_nn_tc<T>(m, n1, n2, A1, lda, tmp, n1, A2, err, s, use_bf16<T>(o));
        } else {
            proj_tn<T>(m, n1, n2, A1, A2, lda, P, tmp, n1, T(0), cnt, err, s);
            update_nn<T>(m, n1, n2, A1, lda, tmp, n1, A2, s);
        }
        int blocks = (int)std::min<int64_t>(ceil_div(n1 * n2, 256), 1024);
        launch_pdl(axpy_block<T>, dim3(blocks), dim3(256), 0, s, (int)n1, (int)n2, (const T*)tmp, (int64_t)n1, R12,
                   ldr);
        log_launch(kTagAxpy, s);
    }
    if (cudaMemset2DAsync(R + n1, ldr * sizeof(T), 0, n2 * sizeof(T), n1, s) != cudaSuccess) return TSQR_ERR_CUDA;
    st = qr_rec<T>(m, n2, A2, lda, R22, ldr, ws, w, o, s);
    if (st != TSQR_OK) return st;
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Blocked Householder QR (tsqr_opts.algorithm = TSQR_QR_HOUSEHOLDER): each
// b-column panel is factored by TSQR, its Householder vectors are
// reconstructed from the explicit panel Q (Ballard, Demmel, Grigori,
// Jacquelin, Knight, Nguyen, "Reconstructing Householder vectors from
// tall-skinny QR", 2015): Q_p - [S; 0] = Y U by an LU without pivoting whose
// signs S = -sign(diagonal) keep every pivot at least 1 in magnitude, and
// T = -U S Y_1^-T gives H_p = I - Y T Y^T with H_p[:, :b] = Q_p S.  The
// trailing columns get H_p^T A2 = A2 - Y (T^T (Y^T A2)) (two GEMMs), and Q is
// accumulated backwards, Q = H_1 ... H_P [I; 0], as LAPACK's orgqr does.
// Orthogonality is then independent of the condition number, unlike the
// block Gram-Schmidt recursion of the reference (block_QR.h:72-95).
// ---------------------------------------------------------------------------
constexpr int kHrMax = 32;  // panel width limit of the Householder path

// Reconstruction of one panel, one CTA.  In: the top bw x bw block of the
// panel's explicit Q (at Ap, lda) and its TSQR factor Rp (bw x bw, ldrp).
// Out: the top block rewritten as the unit lower triangular Y_1, U^-1
// (ld kHrMax), T (bw x bw at Tp, ld ldt) and R_h = S Rp into Rout (upper
// triangle, ldr).
template <typename T>
__global__ void __launch_bounds__(256) hr_reconstruct(int bw, T* Ap, int64_t lda, const T* Rp, int ldrp, T* Uinv,
                                                      T* Tp, int64_t ldt, T* Rout, int64_t ldr) {
    pdl_begin();
    __shared__ T W[kHrMax][kHrMax + 1];   // LU in place: U on and above, L below the diagonal
    __shared__ T Ui[kHrMax][kHrMax + 1];  // U^-1
    __shared__ T Li[kHrMax][kHrMax + 1];  // Y_1^-1 (unit lower)
    __shared__ T sgn[kHrMax];
    const int tid = threadIdx.x;
    for (int e = tid; e < bw * bw; e += blockDim.x) {
        const int i = e % bw, j = e / bw;
        W[i][j] = Ap[i + (int64_t)j * lda];
    }
    __syncthreads();
    for (int i = 0; i < bw; ++i) {
        if (tid == 0) {
            const T s = (W[i][i] >= T(0)) ? T(-1) : T(1);
            sgn[i] = s;
            W[i][i] -= s;
        }
        __syncthreads();
        for (int r = i + 1 + tid; r < bw; r += blockDim.x) {
            const T l = W[r][i] / W[i][i];
            W[r][i] = l;
            for (int c = i + 1; c < bw; ++c) W[r][c] -= l * W[i][c];
        }
        __syncthreads();
    }
    // U^-1 column c by back substitution; Y_1^-1 column c by forward substitution
    for (int c = tid; c < bw; c += blockDim.x) {
        for (int i = c; i >= 0; --i) {
            T x = (i == c) ? T(1) : T(0);
            for (int k = i + 1; k <= c; ++k) x -= W[i][k] * Ui[k][c];
            Ui[i][c] = x / W[i][i];
        }
        for (int i = 0; i < bw; ++i) {
            T z = (i == c) ? T(1) : T(0);
            for (int k = c; k < i; ++k) z -= W[i][k] * Li[k][c];
            Li[i][c] = (i < c) ? T(0) : z;
        }
    }
    __syncthreads();
    for (int e = tid; e < bw * bw; e += blockDim.x) {
        const int i = e % bw, j = e / bw;
        // T = -U S Y_1^-T: sum over i <= k <= j of U(i,k) s_k Y_1^-1(j,k)
        T t = T(0);
        for (int k = i; k <= j; ++k) t -= W[i][k] * sgn[k] * Li[j][k];
        Tp[i + (int64_t)j * ldt] = t;
        Uinv[i + j * kHrMax] = (i <= j) ? Ui[i][j] : T(0);
    }
    for (int e = tid; e < bw * bw; e += blockDim.x) {
        const int i = e % bw, j = e / bw;
        Ap[i + (int64_t)j * lda] = (i > j) ? W[i][j] : ((i == j) ? T(1) : T(0));
        if (i <= j) Rout[i + (int64_t)j * ldr] = sgn[i] * Rp[i + j * ldrp];
    }
}

// Rows of the panel below its top block: y_r = q_r U^-1 (U^-1 upper
// triangular), in place, one thread per row.
template <typename T>
__global__ void __launch_bounds__(256) rows_times_uinv(int64_t rows, int bw, T* Y, int64_t lda, const T* Uinv) {
    pdl_begin();
    __shared__ T U[kHrMax][kHrMax];
    for (int e = threadIdx.x; e < kHrMax * kHrMax; e += blockDim.x) {
        const int i = e % kHrMax, j = e / kHrMax;
        U[i][j] = (i < bw && j < bw) ? Uinv[i + j * kHrMax] : T(0);
    }
    __syncthreads();
    // compile-time bounds keep the row in registers; columns past bw are zero
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        T q[kHrMax];
#pragma unroll
        for (int k = 0; k < kHrMax; ++k) q[k] = (k < bw) ? Y[r + (int64_t)k * lda] : T(0);
#pragma unroll
        for (int c = 0; c < kHrMax; ++c) {
            T y = T(0);
#pragma unroll
            for (int k = 0; k <= c; ++k) y = fma(q[k], U[k][c], y);
            if (c < bw) Y[r + (int64_t)c * lda] = y;
        }
    }
}

// Products with an upper triangular U (ld ldu), one thread per output:
//   kind 0: X = alpha U^T W   (p x q; U is p x p)
//   kind 1: X = alpha U W     (p x q; U is p x p)
//   kind 2: X = alpha W U     (p x q; U is q x q)
template <typename T>
__global__ void tri_mul(int kind, int p, int64_t q, const T* U, int64_t ldu, const T* W, int64_t ldw, T alpha, T* X,
                        int64_t ldx) {
    pdl_begin();
    const int64_t total = (int64_t)p * q;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % p);
        const int64_t c = e / p;
        T x = T(0);
        if (kind == 0)
            for (int k = 0; k <= i; ++k) x = fma(U[k + (int64_t)i * ldu], W[k + c * ldw], x);
        else if (kind == 1)
            for (int k = i; k < p; ++k) x = fma(U[i + (int64_t)k * ldu], W[k + c * ldw], x);
        else
            for (int64_t k = 0; k <= c; ++k) x = fma(W[i + k * ldw], U[k + c * ldu], x);
        X[i + c * ldx] = alpha * x;
    }
}

// M = T Y_1^T (bw x bw, ld kHrMax) for the panel's columns of Q, one CTA: T
// upper (ld ldt) and Y_1 unit lower, so M(i, c) = sum over i <= k <= c of
// T(i,k) Y_1(c,k).
template <typename T>
__global__ void panel_m(int bw, const T* Y, int64_t lda, const T* Tp, int64_t ldt, T* M) {
    pdl_begin();
    for (int e = threadIdx.x; e < bw * bw; e += blockDim.x) {
        const int i = e % bw, c = e / bw;
        T x = T(0);
        for (int k = i; k <= c; ++k) x = fma(Tp[i + (int64_t)k * ldt], Y[c + (int64_t)k * lda], x);
        M[i + c * kHrMax] = x;
    }
}

// The panel's columns of Q: row r of [I; 0] - Y M, in place over Y, one
// thread per row (each row reads only itself).
template <typename T>
__global__ void __launch_bounds__(256) panel_q_rows(int64_t rows, int bw, T* Y, int64_t lda, const T* M) {
    pdl_begin();
    __shared__ T Ms[kHrMax][kHrMax + 1];
    for (int e = threadIdx.x; e < kHrMax * kHrMax; e += blockDim.x) {
        const int i = e % kHrMax, j = e / kHrMax;
        Ms[i][j] = (i < bw && j < bw) ? M[i + j * kHrMax] : T(0);
    }
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
        T y[kHrMax];
#pragma unroll
        for (int k = 0; k < kHrMax; ++k) y[k] = (k < bw) ? Y[r + (int64_t)k * lda] : T(0);
#pragma unroll
        for (int c = 0; c < kHrMax; ++c) {
            T q = (r == c) ? T(1) : T(0);
#pragma unroll
            for (int k = 0; k < kHrMax; ++k) q = fma(-y[k], Ms[k][c], q);
            if (c < bw) Y[r + (int64_t)c * lda] = q;
        }
    }
}

// The Householder path is recursive, like the block Gram-Schmidt one: the
// left half is factored, H_1^T is applied to the right half with one GEMM
// pair of inner dimension n1, the right half's lower rows are factored, and
// the two compact-WY factors combine, T = [T1, -T1 (Y1^T Y2) T2; 0, T2].  Q
// is formed the same way backwards.  Every large product is a GEMM of inner
// dimension >= the panel width, so the tensor-core form applies to it as to
// block Gram-Schmidt.  Leaves (n <= panel) are TSQR + reconstruction.
//
// Workspace: [status word | leaf TSQR | split-K partials | Rp, U^-1, M of a
// leaf | W, X (n1 x n2 each) | T of the whole matrix (n x n)].
struct HqrWs {
    size_t err = kPHeader, tsqr = 0, part = 0, small = 0, wx = 0, tfull = 0;
    size_t total() const { return err + tsqr + part + small + wx + tfull; }
};

template <typename T>
void hqr_ws_walk(int64_t m, int64_t n, int b, bool tc, HqrWs* w) {
    if (n <= b) {
        const size_t tb = tc ? tsqr_precision_workspace(m, n) : tsqr_plain_workspace<T>(m, n);
        w->tsqr = std::max(w->tsqr, (size_t)round_up((int64_t)tb, 256));
        return;
    }
    const int64_t n1 = split_of(n, b), n2 = n - n1;
    for (int64_t K : {m, m - n1}) {
        const size_t pb = tc_projection(tc, n1, n2) ? (size_t)tc_tn_splits(n1, n2, K) * n1 * n2 * sizeof(T)
                                                    : proj_tn_part_bytes<T>(n1, n2, K);
        w->part = std::max(w->part, (size_t)round_up((int64_t)pb, 256));
    }
    w->wx = std::max(w->wx, 2 * (size_t)round_up(n1 * n2 * (int64_t)sizeof(T), 256));
    hqr_ws_walk<T>(m, n1, b, tc, w);
    hqr_ws_walk<T>(m - n1, n2, b, tc, w);
}

template <typename T>
HqrWs hqr_ws(int64_t m, int64_t n, int b, bool tc) {
    HqrWs w;
    hqr_ws_walk<T>(m, n, b, tc, &w);
    w.small = 3 * (size_t)round_up((int64_t)(b * b * sizeof(T)), 256);
    w.tfull = (size_t)round_up(n * n * (int64_t)sizeof(T), 256);
    return w;
}

template <typename T>
struct HqrCtx {
    int64_t lda, ldr, ldt;
    char* tws;
    size_t tsqr_bytes;
    T *part, *Rp, *Uinv, *Mb, *W, *X;
    int* err;
    bool tc;
    bool bf16 = false;  // BF16x3 tensor-core GEMMs
    int b;
    cudaStream_t s;
};

inline unsigned grid_of(int64_t work, int64_t cap) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(work, 256), cap));
}

// C (n1 x n2, ld n1) = A1^T A2 over m rows (A1, A2 share lda)
template <typename T>
void hqr_tn(const HqrCtx<T>& c, int64_t m, int64_t n1, int64_t n2, const T* A1, const T* A2, T* C) {
    if (tc_projection(c.tc, n1, n2))
        proj_tn_tc<T>(m, n1, n2, A1, A2, c.lda, c.part, C, n1, T(0), c.err, c.s, c.bf16);
    else
        proj_tn<T>(m, n1, n2, A1, A2, c.lda, c.part, C, n1, T(0), c.err + kPCounters, c.err, c.s);
}

// A2 (m x n2) -= Y (m x n1) X (n1 x n2, ld n1)
template <typename T>
void hqr_nn(const HqrCtx<T>& c, int64_t m, int64_t n1, int64_t n2, const T* Y, const T* X, T* A2) {
    if (c.tc) {
        update_nn_tc<T>(m, n1, n2, Y, c.lda, X, n1, A2, c.err, c.s, c.bf16);
    } else {
        update_nn<T>(m, n1, n2, Y, c.lda, X, n1, A2, c.s);
    }
}

// Factor the m x n block A (rows and columns from its own origin): Y below
// its diagonal, R into Rb, T into Tb (ld ldt).
template <typename T>
tsqr_status hqr_factor(const HqrCtx<T>& c, int64_t m, int64_t n, T* A, T* Rb, T* Tb) {
    if (n <= c.b) {
        tsqr_status st;
        if constexpr (std::is_same<T, float>::value) {
            st = c.tc ? tsqr_precision(m, n, A, c.lda, c.Rp, n, c.tws, c.tsqr_bytes, c.s)
                      : tsqr_plain<T>(m, n, A, c.lda, c.Rp, n, c.tws, c.tsqr_bytes, c.s);
        } else {
            st = tsqr_plain<T>(m, n, A, c.lda, c.Rp, n, c.tws, c.tsqr_bytes, c.s);
        }
        if (st != TSQR_OK) return st;
        hr_reconstruct<T><<<1, 256, 0, c.s>>>((int)n, A, c.lda, c.Rp, (int)n, c.Uinv, Tb, c.ldt, Rb, c.ldr);
        log_launch(kTagHouse, c.s);
        if (m > n) {
            rows_times_uinv<T><<<grid_of(m - n, 4096), 256, 0, c.s>>>(m - n, (int)n, A + n, c.lda, c.Uinv);
            log_launch(kTagHouse + 1, c.s);
        }
        return TSQR_OK;
    }
    const int64_t n1 = split_of(n, c.b), n2 = n - n1;
    T* A2 = A + n1 * c.lda;
    tsqr_status st = hqr_factor<T>(c, m, n1, A, Rb, Tb);
    if (st != TSQR_OK) return st;
    // A2 <- H_1^T A2 = A2 - Y1 (T1^T (Y1^T A2))
    hqr_tn<T>(c, m, n1, n2, A, A2, c.W);
    tri_mul<T><<<grid_of(n1 * n2, 1024), 256, 0, c.s>>>(0, (int)n1, n2, Tb, c.ldt, c.W, n1, T(1), c.X, n1);
    log_launch(kTagHouse + 2, c.s);
    hqr_nn<T>(c, m, n1, n2, A, c.X, A2);
    if (cudaMemcpy2DAsync(Rb + n1 * c.ldr, c.ldr * sizeof(T), A2, c.lda * sizeof(T), n1 * sizeof(T), n2,
                          cudaMemcpyDeviceToDevice, c.s) != cudaSuccess)
        return TSQR_ERR_CUDA;
    // R12 now lives in R; zeroing it here leaves Y of this block (leaf Y's
    // with zeros above their unit diagonals) clean for every later product
    if (cudaMemset2DAsync(A2, c.lda * sizeof(T), 0, n1 * sizeof(T), n2, c.s) != cudaSuccess) return TSQR_ERR_CUDA;
    T* Tb2 = Tb + n1 + n1 * c.ldt;
    st = hqr_factor<T>(c, m - n1, n2, A2 + n1, Rb + n1 + n1 * c.ldr, Tb2);
    if (st != TSQR_OK) return st;
    // T12 = -T1 (Y1^T Y2) T2, Y2 living in rows n1.. of the block
    hqr_tn<T>(c, m - n1, n1, n2, A + n1, A2 + n1, c.W);
    tri_mul<T><<<grid_of(n1 * n2, 1024), 256, 0, c.s>>>(2, (int)n1, n2, Tb2, c.ldt, c.W, n1, T(1), c.X, n1);
    tri_mul<T><<<grid_of(n1 * n2, 1024), 256, 0, c.s>>>(1, (int)n1, n2, Tb, c.ldt, c.X, n1, T(-1), Tb + n1 * c.ldt,
                                                         c.ldt);
    log_launch(kTagHouse + 2, c.s);
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

// Q of the m x n block from its Y (in A) and T (Tb): Q = H [I; 0], in place.
template <typename T>
tsqr_status hqr_form_q(const HqrCtx<T>& c, int64_t m, int64_t n, T* A, const T* Tb) {
    if (n <= c.b) {
        panel_m<T><<<1, 256, 0, c.s>>>((int)n, A, c.lda, Tb, c.ldt, c.Mb);
        panel_q_rows<T><<<grid_of(m, 4096), 256, 0, c.s>>>(m, (int)n, A, c.lda, c.Mb);
        log_launch(kTagHouse + 3, c.s);
        return TSQR_OK;
    }
    const int64_t n1 = split_of(n, c.b), n2 = n - n1;
    T* A2 = A + n1 * c.lda;
    // right half first: Q2 = H_2 [I; 0] in rows n1.., zeros above it
    tsqr_status st = hqr_form_q<T>(c, m - n1, n2, A2 + n1, Tb + n1 + n1 * c.ldt);
    if (st != TSQR_OK) return st;
    if (cudaMemset2DAsync(A2, c.lda * sizeof(T), 0, n1 * sizeof(T), n2, c.s) != cudaSuccess) return TSQR_ERR_CUDA;
    // then H_1 applied to it: A2 - Y1 (T1 (Y1^T A2))
    hqr_tn<T>(c, m, n1, n2, A, A2, c.W);
    tri_mul<T><<<grid_of(n1 * n2, 1024), 256, 0, c.s>>>(1, (int)n1, n2, Tb, c.ldt, c.W, n1, T(1), c.X, n1);
    log_launch(kTagHouse + 2, c.s);
    hqr_nn<T>(c, m, n1, n2, A, c.X, A2);
    // the left half last: its Y1 was needed above
    return hqr_form_q<T>(c, m, n1, A, Tb);
}

template <typename T>
tsqr_status hqr_run(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                    const tsqr_opts& o, cudaStream_t s) {
    const int b = panel_of(o);
    if (b > kHrMax) return TSQR_ERR_UNSUPPORTED;
    const bool tc = use_tc<T>(o);
    const HqrWs w = hqr_ws<T>(m, n, b, tc);
    if (work == nullptr || work_bytes < w.total()) return TSQR_ERR_WORKSPACE;
    char* base = static_cast<char*>(work);
    HqrCtx<T> c;
    c.lda = lda;
    c.ldr = ldr;
    c.ldt = n;
    c.err = reinterpret_cast<int*>(base);
    c.tws = base + w.err;
    c.tsqr_bytes = w.tsqr;
    c.part = reinterpret_cast<T*>(c.tws + w.tsqr);
    const size_t bb = (size_t)round_up((int64_t)(b * b * sizeof(T)), 256);
    char* sm = c.tws + w.tsqr + w.part;
    c.Rp = reinterpret_cast<T*>(sm);
    c.Uinv = reinterpret_cast<T*>(sm + bb);
    c.Mb = reinterpret_cast<T*>(sm + 2 * bb);
    c.W = reinterpret_cast<T*>(sm + w.small);
    c.X = reinterpret_cast<T*>(sm + w.small + w.wx / 2);
    T* Tfull = reinterpret_cast<T*>(sm + w.small + w.wx);
    c.tc = tc;
    c.bf16 = use_bf16<T>(o);
    c.b = b;
    c.s = s;
    // status word and the projection's counters
    if (cudaMemsetAsync(c.err, 0, kPHeader, s) != cudaSuccess) return TSQR_ERR_CUDA;
    if (cudaMemset2DAsync(R, ldr * sizeof(T), 0, n * sizeof(T), n, s) != cudaSuccess) return TSQR_ERR_CUDA;
    if (cudaMemsetAsync(Tfull, 0, n * n * sizeof(T), s) != cudaSuccess) return TSQR_ERR_CUDA;
    tsqr_status st = hqr_factor<T>(c, m, n, A, R, Tfull);
    if (st != TSQR_OK) return st;
    return hqr_form_q<T>(c, m, n, A, Tfull);
}

}  // namespace

template <typename T>
size_t qr_workspace(int64_t m, int64_t n, const tsqr_opts& o) {
    if (o.algorithm == TSQR_QR_HOUSEHOLDER)
        return panel_of(o) <= kHrMax ? hqr_ws<T>(m, n, panel_of(o), use_tc<T>(o)).total() : 0;
    QrWs w;
    qr_ws_walk<T>(m, n, panel_of(o), o.reorth != 0, use_tc<T>(o), &w);
    return w.total();
}

template <typename T>
tsqr_status qr_run(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                   const tsqr_opts& o, cudaStream_t s) {
    if (o.algorithm == TSQR_QR_HOUSEHOLDER) return hqr_run<T>(m, n, A, lda, R, ldr, work, work_bytes, o, s);
    QrWs w;
    qr_ws_walk<T>(m, n, panel_of(o), o.reorth != 0, use_tc<T>(o), &w);
    if (work == nullptr || work_bytes < w.total()) return TSQR_ERR_WORKSPACE;
    // status word and the projection's counters
    if (cudaMemsetAsync(work, 0, kPHeader, s) != cudaSuccess) return TSQR_ERR_CUDA;
    return qr_rec<T>(m, n, A, lda, R, ldr, reinterpret_cast<char*>(work), w, o, s);
}

template size_t qr_workspace<float>(int64_t, int64_t, const tsqr_opts&);
template size_t qr_workspace<double>(int64_t, int64_t, const tsqr_opts&);
template tsqr_status qr_run<float>(int64_t, int64_t, float*, int64_t, float*, int64_t, void*, size_t,
                                   const tsqr_opts&, cudaStream_t);
template tsqr_status qr_run<double>(int64_t, int64_t, double*, int64_t, double*, int64_t, void*, size_t,
                                    const tsqr_opts&, cudaStream_t);

}  // namespace tsqr
