// tsqr_kernels.cuh -- CUDA-core (plain precision) TSQR tile kernels.
//
// A "level matrix" M (h x n, column-major, leading dimension ld) is cut into
// tiles of B = NT*RPT rows.  Level 0 is the caller's A; level l+1 stacks the
// n x n R factors of level l's tiles (h_{l+1} = tiles_l * n); the level with
// a single tile is the root.  This is the reduction tree of the reference's
// persistent tsqr_kernel (kernelQR.h:341-388) and of its two-level chunk
// scheme (TallShinnyQR.h:106-127), restated as one tree with a tile height
// chosen per (dtype, n) instead of the compile-time BLOCK_SIZE=128 and
// NUM_SM=108 (kernelQR.h:3-4).
//
// factor_tiles: Householder QR of each tile (the reference's qr_kernel,
//   kernelQR.h:69-220), LAPACK larfg form: H_j = I - tau_j v_j v_j^T with
//   v_j(j) = 1 and R_jj = beta_j = -sign(alpha) ||x||, the same diagonal sign
//   rule as kernelQR.h:139-142.  Instead of forming the tile's explicit Q in
//   shared memory (kernelQR.h:224-290) it leaves the compact-WY form in place:
//   the strict lower part of the tile holds V, the upper triangle of the
//   tile's top n x n block holds T (H_0...H_{n-1} = I - V T V^T).  The tile
//   lives in registers (RPT rows x NMAX columns per thread).  Each column
//   costs two block barriers: one after the norm partials, one after the
//   dot-product partials (the warp transpose-reduction of NMAX values, then a
//   redundant per-warp finalisation instead of a third barrier).  The same
//   reduction also yields column j of V^T V, from which T is formed once per
//   tile: row i of T depends only on row i (T(i,j) = -tau_j sum_k T(i,k)
//   S(k,j)), so thread i builds it alone.  R goes to the next level's rows
//   [t*n, t*n+n), or to the caller's R at the root.  With NORM64 the norm,
//   beta and tau are computed in FP64.
//
// apply_tiles: down-sweep (kernelQR.h:397-492 and tsgemm_tsqr,
//   TallShinnyQR.h:11-74): given the parent's n x n block B_t (the root uses
//   B = I), the tile's final Q is (I - V T V^T) [B_t; 0] = [B_t; 0] - V W,
//   W = T (V_top^T B_t).  W needs only the tile's top block, so the bulk is a
//   reduction-free (B x n)(n x n) product streamed as n rank-1 updates of
//   each thread's rows; Q overwrites the tile in place.
//
// Rows of the last tile past the matrix end are treated as zero rows: they
// never change, never enter a dot product and are never stored.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace tsqr {

template <typename T>
struct FactorParams {
    T* M;           // level matrix (tiles are factored in place)
    int64_t ld;
    int64_t h;      // rows of the level matrix
    int n;
    int64_t ntiles;
    T* Rout;        // R of tile t goes to rows [t*n, t*n+n) of Rout
    int64_t ldr;
};

template <typename T>
struct ApplyParams {
    T* M;
    int64_t ld;
    int64_t h;
    int n;
    int64_t ntiles;
    const T* P;     // parent level's final Q (rows t*n.. of tile t); null = identity
    int64_t ldp;
    int vec;        // 1: ld and the level base allow 16-byte copies
};

// Shared memory of one factor CTA.
template <typename T, int NMAX, int NT, bool NORM64>
struct FactorSmem {
    static constexpr int NW = NT / 32;
    using N64 = typename std::conditional<NORM64, double, T>::type;
    N64 s_part[NW];
    T s_alpha;
    T red[NW][NMAX];
    __align__(16) T wfin[NW][NMAX];
    T Ssh[NMAX][NMAX + 1];
    T Tsh[NMAX][NMAX + 1];
    T tau_sh[NMAX];
    T rdiag[NMAX];
    // per-warp transpose scratch of the FP32 dot-product reduction
    __align__(16) float xpose[std::is_same<T, float>::value ? NW : 1]
                             [std::is_same<T, float>::value ? 32 * xpose_stride<NMAX>() : 4];
};

// Householder QR of one tile: ht (<= NT*RPT) rows of n columns at `tile`
// (leading dimension ld), factored in place (V below the diagonal, T in the
// top block's upper triangle); its n x n R goes to Rt (leading dimension
// ldr).  Called by every thread of the CTA.
template <typename T, int NMAX, int NT, int RPT, bool NORM64>
__device__ __forceinline__ void factor_tile(FactorSmem<T, NMAX, NT, NORM64>& S, T* tile, int64_t ld, int ht, int n,
                                            T* Rt, int64_t ldr) {
    constexpr int NW = NT / 32;
    constexpr int U = 4;  // columns per unrolled group
    static_assert(NT >= NMAX && NT % 32 == 0 && NMAX % U == 0, "bad tile configuration");
    using N64 = typename FactorSmem<T, NMAX, NT, NORM64>::N64;
    auto& s_part = S.s_part;
    auto& s_alpha = S.s_alpha;
    auto& red = S.red;
    auto& wfin = S.wfin;
    auto& Ssh = S.Ssh;
    auto& Tsh = S.Tsh;
    auto& tau_sh = S.tau_sh;
    auto& rdiag = S.rdiag;
    auto& xpose = S.xpose;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = (n + U - 1) / U;
    const int shift = (U * G) % NMAX;  // register position c ends up holding column (c + shift) % NMAX
    {
        // y[i][c]: row tid + NT*i.  The column loop runs in groups of U
        // columns; after each group the register row rotates left by U, so at
        // group g position c < n - U*g holds column U*g + c (positions 0..U-1
        // are the group's columns) and position NMAX - U*g + k holds the
        // finished reflector v_k.  All register indices stay compile-time
        // while the code holds U column steps instead of NMAX.
        T y[RPT][NMAX];
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = tid + NT * i;
#pragma unroll
            for (int c = 0; c < NMAX; ++c)
                y[i][c] = (r < ht && c < n) ? tile[r + c * ld] : T(0);
        }

#pragma unroll 1
        for (int g = 0; g < G; ++g) {
            const int base = U * g;
            const int live = n - base;      // positions [0, live): columns base .. n-1
            const int past0 = NMAX - base;  // positions [past0, NMAX): v_0 .. v_{base-1}
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int j = base + u;
                if (j < n) {
                    // Row slots i >= 1 hold rows >= NT >= NMAX > j, so only
                    // slot 0 needs the row-versus-diagonal tests below.
                    // (a) sigma^2 = ||x(j+1:, j)||^2 and alpha = x(j, j)
                    N64 s = 0;
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const int r = tid + NT * i;
                        if (i > 0 || r > j) s += (N64)y[i][u] * (N64)y[i][u];
                        if (i == 0 && r == j) s_alpha = y[i][u];
                    }
                    s = warp_sum(s);
                    if (lane == 0) s_part[warp] = s;
                    __syncthreads();
                    N64 sigma2 = 0;
#pragma unroll
                    for (int w = 0; w < NW; ++w) sigma2 += s_part[w];
                    const N64 alpha = s_alpha;
                    N64 beta, tau, scale;
                    if (sigma2 == N64(0)) {
                        tau = 0;
                        beta = alpha;
                        scale = 0;
                    } else {
                        const N64 nrm = sqrt(alpha * alpha + sigma2);
                        beta = (alpha >= N64(0)) ? -nrm : nrm;
                        // reciprocal-multiply (round-to-nearest reciprocal)
                        // keeps the slow division path off the column chain
                        tau = (beta - alpha) * recip(beta);
                        scale = recip(alpha - beta);
                    }
                    const T taut = (T)tau;
                    const T scalet = (T)scale;
                    // (b) v_j below the diagonal (v_j(j) = 1 implicitly), then
                    // v_j . y[c] for every other position: trailing columns
                    // (update) and finished reflectors (column j of V^T V)
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const int r = tid + NT * i;
                        if (i > 0 || r > j) y[i][u] *= scalet;
                    }
                    // v of slot 0: 0 above the diagonal, 1 on it
                    const T v0 = (tid > j) ? y[0][u] : ((tid == j) ? T(1) : T(0));
                    T pc[NMAX];
#pragma unroll
                    for (int c = 0; c < NMAX; ++c) pc[c] = (c != u) ? v0 * y[0][c] : T(0);
#pragma unroll
                    for (int i = 1; i < RPT; ++i) {
                        const T v = y[i][u];
#pragma unroll
                        for (int c = 0; c < NMAX; ++c)
                            if (c != u) pc[c] += v * y[i][c];
                    }
                    if constexpr (std::is_same<T, float>::value)
                        warp_reduce_to_smem_x<NMAX>(pc, red[warp], xpose[warp], lane);
                    else
                        warp_reduce_to_smem<T, NMAX>(pc, red[warp], lane);
                    __syncthreads();
                    // (c) every warp sums the NW partials itself; positions
                    // that are not trailing columns get a zero coefficient, so
                    // the update below needs no per-column test
                    {
                        constexpr int K = NMAX >= 32 ? NMAX / 32 : 1;
#pragma unroll
                        for (int kk = 0; kk < K; ++kk) {
                            const int idx = (NMAX >= 32) ? lane * K + kk : lane;
                            if (idx < NMAX) {
                                T a = 0;
#pragma unroll
                                for (int w = 0; w < NW; ++w) a += red[w][idx];
                                wfin[warp][idx] = (idx > u && idx < live) ? a : T(0);
                                if (warp == 0) {
                                    const int k = (idx >= past0) ? idx - past0 : ((idx < u) ? base + idx : -1);
                                    if (k >= 0) Ssh[k][j] = a;
                                }
                            }
                        }
                        if (tid == 0) {
                            tau_sh[j] = taut;
                            rdiag[j] = (T)beta;
                        }
                    }
                    __syncwarp();
                    // (d) trailing update x_c -= tau (v^T x_c) v (v = 0 above
                    // the diagonal, coefficient 0 off the trailing columns)
                    T wr[NMAX];
#pragma unroll
                    for (int c = 0; c < NMAX; ++c) wr[c] = wfin[warp][c];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const T tv = taut * ((i > 0) ? y[i][u] : v0);
#pragma unroll
                        for (int c = u + 1; c < NMAX; ++c) y[i][c] -= tv * wr[c];
                    }
                }
            }
            // rotate every register row left by U
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                T keep[U];
#pragma unroll
                for (int u = 0; u < U; ++u) keep[u] = y[i][u];
#pragma unroll
                for (int c = 0; c < NMAX - U; ++c) y[i][c] = y[i][c + U];
#pragma unroll
                for (int u = 0; u < U; ++u) y[i][NMAX - U + u] = keep[u];
            }
        }
        __syncthreads();  // Ssh, tau_sh, rdiag complete

        // T, one row per thread: T(i,i) = tau_i,
        // T(i,j) = -tau_j sum_{k=i}^{j-1} T(i,k) S(k,j) for j > i.
        if (tid < n) {
            const int i = tid;
            T trow[NMAX];
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                T val = T(0);
                if (j == i) {
                    val = tau_sh[j];
                } else if (j > i && j < n) {
                    T a = 0;
#pragma unroll
                    for (int k = 0; k < j; ++k)
                        if (k >= i) a += trow[k] * Ssh[k][j];
                    val = -tau_sh[j] * a;
                }
                trow[j] = val;
            }
#pragma unroll
            for (int j = 0; j < NMAX; ++j) Tsh[i][j] = trow[j];
        }
        __syncthreads();

        // R of this tile: row r < n is held by thread r (i = 0).
        if (tid < n) {
            const int r = tid;
#pragma unroll
            for (int c = 0; c < NMAX; ++c) {
                const int k = (c + shift) % NMAX;
                if (k < n) {
                    T v = (k > r) ? y[0][c] : ((k == r) ? rdiag[r] : T(0));
                    if (r >= ht) v = T(0);
                    Rt[r + k * ldr] = v;
                }
            }
        }
        // V below the diagonal, T in the top block's upper triangle.
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = tid + NT * i;
            if (r < ht) {
#pragma unroll
                for (int c = 0; c < NMAX; ++c) {
                    const int k = (c + shift) % NMAX;
                    if (k < n) tile[r + k * ld] = (r > k) ? y[i][c] : Tsh[r][k];
                }
            }
        }
        __syncthreads();
    }
}

template <typename T, int NMAX, int NT, int RPT, int MINB, bool NORM64>
__global__ void __launch_bounds__(NT, MINB) factor_tiles(FactorParams<T> p) {
    constexpr int B = NT * RPT;
    __shared__ FactorSmem<T, NMAX, NT, NORM64> S;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int64_t row0 = t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        factor_tile<T, NMAX, NT, RPT, NORM64>(S, p.M + row0, p.ld, ht, p.n, p.Rout + t * p.n, p.ldr);
    }
}

template <typename T, int NMAX, int B>
constexpr size_t apply_smem_bytes() {
    // Vs: the tile (NMAX x B, ld B), Ws: NMAX x NMAX, Vt/Tt/Bs/Ys: NMAX x (NMAX+1)
    return sizeof(T) * ((size_t)NMAX * B + (size_t)NMAX * NMAX + 4 * (size_t)NMAX * (NMAX + 1));
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Q assembly of one tile: ht (<= NT*RPT) rows of n columns at `tile` (ld),
// holding V and T from factor_tile, overwritten by (I - V T V^T) [B; 0]
// where B is the n x n block at Pb (leading dimension ldp), or the identity
// when Pb is null.  vec: 16-byte copies are legal (ld and tile aligned).
// smem: apply_smem_bytes<T, NMAX, NT*RPT>() bytes.  Called by every thread.
template <typename T, int NMAX, int NT, int RPT>
__device__ __forceinline__ void apply_tile(unsigned char* apply_smem, T* tile, int64_t ld, int ht, int n,
                                           const T* Pb, int64_t ldp, int vec) {
    constexpr int B = NT * RPT;
    constexpr int VE = 16 / sizeof(T);  // elements per 16-byte copy
    typedef T Row1[NMAX + 1];
    typedef T Row0[NMAX];
    T* Vs = reinterpret_cast<T*>(apply_smem);
    Row0* Ws = reinterpret_cast<Row0*>(Vs + (size_t)NMAX * B);
    Row1* Vt = reinterpret_cast<Row1*>(Ws + NMAX);
    Row1* Tt = Vt + NMAX;
    Row1* Bs = Tt + NMAX;
    Row1* Ys = Bs + NMAX;
    const int tid = threadIdx.x;
    struct {
        int64_t ld, ldp;
        const T* P;
        int vec;
    } p = {ld, ldp, Pb, vec};
    const int64_t t = 0;  // Pb already points at this tile's block
    {
        // Stage the whole tile into shared memory with asynchronous copies;
        // they land while the top-block products below are computed.
        if (p.vec) {
            constexpr int NV = B / VE;
            for (int e = tid; e < n * NV; e += NT) {
                const int c = e / NV, r = (e % NV) * VE;
                if (r + VE <= ht) {
                    cp_async<16>(Vs + (size_t)c * B + r, tile + r + (int64_t)c * p.ld);
                } else {
                    for (int rr = r; rr < ht; ++rr)
                        cp_async<sizeof(T)>(Vs + (size_t)c * B + rr, tile + rr + (int64_t)c * p.ld);
                }
            }
        } else {
            for (int e = tid; e < n * B; e += NT) {
                const int c = e / B, r = e % B;
                if (r < ht) cp_async<sizeof(T)>(Vs + (size_t)c * B + r, tile + r + (int64_t)c * p.ld);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");

        for (int idx = tid; idx < NMAX * NMAX; idx += NT) {
            const int r = idx % NMAX, c = idx / NMAX;
            const bool in = (r < ht && r < n && c < n);
            const T v = in ? tile[r + c * p.ld] : T(0);
            Vt[r][c] = (r > c) ? v : ((r == c && c < n) ? T(1) : T(0));
            Tt[r][c] = (r <= c) ? v : T(0);
            T b;
            if (p.P)
                b = (r < n && c < n) ? p.P[t * n + r + c * p.ldp] : T(0);
            else
                b = (r == c && r < n) ? T(1) : T(0);
            Bs[r][c] = b;
        }
        __syncthreads();
        // Y = V_top^T B (V_top is unit lower triangular: terms r >= k)
        for (int idx = tid; idx < NMAX * NMAX; idx += NT) {
            const int k = idx % NMAX, c = idx / NMAX;
            T a = 0;
#pragma unroll
            for (int r = 0; r < NMAX; ++r) a += Vt[r][k] * Bs[r][c];
            Ys[k][c] = a;
        }
        __syncthreads();
        // W = T Y (T upper triangular: its zeros make the full sum exact)
        for (int idx = tid; idx < NMAX * NMAX; idx += NT) {
            const int k = idx % NMAX, c = idx / NMAX;
            T a = 0;
#pragma unroll
            for (int l = 0; l < NMAX; ++l) a += Tt[k][l] * Ys[l][c];
            Ws[k][c] = a;
        }
        cp_async_wait_all();
        __syncthreads();

        // Q rows = [B; 0] - V W as n rank-1 updates of the thread's rows.
        T q[RPT][NMAX];
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = tid + NT * i;
#pragma unroll
            for (int c = 0; c < NMAX; ++c) q[i][c] = (r < n) ? Bs[r][c] : T(0);
        }
#pragma unroll 8
        for (int k = 0; k < NMAX; ++k) {
            if (k < n) {
                T vk[RPT];
#pragma unroll
                for (int i = 0; i < RPT; ++i) {
                    const int r = tid + NT * i;
                    // rows of the top block come masked (T above the
                    // diagonal, unit diagonal); the rest from the staged tile
                    vk[i] = (r < n) ? Vt[r][k] : ((r < ht) ? Vs[(size_t)k * B + r] : T(0));
                }
#pragma unroll
                for (int c = 0; c < NMAX; ++c) {
                    const T w = Ws[k][c];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) q[i][c] -= vk[i] * w;
                }
            }
        }
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            const int r = tid + NT * i;
            if (r < ht) {
#pragma unroll
                for (int c = 0; c < NMAX; ++c)
                    if (c < n) tile[r + c * p.ld] = q[i][c];
            }
        }
        __syncthreads();
    }
}

template <typename T, int NMAX, int NT, int RPT, int MINB>
__global__ void __launch_bounds__(NT, MINB) apply_tiles(ApplyParams<T> p) {
    constexpr int B = NT * RPT;
    extern __shared__ __align__(16) unsigned char apply_smem[];
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int64_t row0 = t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        apply_tile<T, NMAX, NT, RPT>(apply_smem, p.M + row0, p.ld, ht, p.n, p.P ? p.P + t * p.n : nullptr, p.ldp,
                                     p.vec);
    }
}

}  // namespace tsqr
