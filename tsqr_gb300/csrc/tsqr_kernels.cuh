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

#include <cuda.h>  // CUtensorMap (the type only; no driver calls here)

#include "common.cuh"
#include "tc.cuh"

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
    int* err = nullptr;  // status word: set to 1 when a bounded wait gives up (null: none)
    int tries = tc::kMbarTries;  // polls of a bounded wait before it gives up
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

// Column-major V^T V of a tile: Sc[j][k] = S(k, j) = v_k . v_j for k < j,
// rows padded to a multiple of 16 bytes so a column reads as vector loads.
template <typename T, int NMAX>
struct SCols {
    static constexpr int LD = NMAX + 16 / (int)sizeof(T);
    __align__(16) T c[NMAX][LD];
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
    SCols<T, NMAX> Sc;
    T Tsh[NMAX][NMAX + 1];
    T tau_sh[NMAX];
    T rdiag[NMAX];
    // per-warp transpose scratch of the FP32 dot-product reduction
    __align__(16) float xpose[std::is_same<T, float>::value ? NW : 1]
                             [std::is_same<T, float>::value ? 32 * xpose_stride<NMAX>() : 4];
};

// Row i of the compact-WY factor T of a tile: T(i,i) = tau_i and
// T(i,j) = -tau_j sum_{k=i}^{j-1} T(i,k) S(k,j) for i < j < n, zero
// elsewhere.  Column j of S is read with 16-byte loads that do not depend on
// the FMA chain, so their latency is paid once per column instead of once per
// product, and the chain is split into two accumulators.  T(i,k) = 0 for
// k < i, so the sum runs over every k < j without a per-thread test.
template <typename T, int NMAX>
__device__ __forceinline__ void t_factor_row(const SCols<T, NMAX>& S, const T* tau, int i, int n, T (&trow)[NMAX]) {
    constexpr int VW = 16 / (int)sizeof(T);  // elements per 16-byte load
    static_assert(NMAX % VW == 0, "T build reads whole 16-byte groups");
#pragma unroll
    for (int j = 0; j < NMAX; ++j) {
        T a0 = T(0), a1 = T(0);
#pragma unroll
        for (int k0 = 0; k0 < j; k0 += VW) {
            if constexpr (VW == 4) {
                const float4 q = *reinterpret_cast<const float4*>(&S.c[j][k0]);
                a0 += trow[k0] * q.x;
                if (k0 + 1 < j) a1 += trow[k0 + 1] * q.y;
                if (k0 + 2 < j) a0 += trow[k0 + 2] * q.z;
                if (k0 + 3 < j) a1 += trow[k0 + 3] * q.w;
            } else {
                const double2 q = *reinterpret_cast<const double2*>(&S.c[j][k0]);
                a0 += trow[k0] * q.x;
                if (k0 + 1 < j) a1 += trow[k0 + 1] * q.y;
            }
        }
        const T tj = tau[j];
        trow[j] = (j == i) ? tj : ((j > i && j < n) ? -tj * (a0 + a1) : T(0));
    }
}

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
    auto& Sc = S.Sc.c;
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
                                    if (k >= 0) Sc[j][k] = a;
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
        __syncthreads();  // V^T V, tau_sh, rdiag complete

        // T, one row per thread: T(i,i) = tau_i,
        // T(i,j) = -tau_j sum_{k=i}^{j-1} T(i,k) S(k,j) for j > i.
        if (tid < n) {
            const int i = tid;
            T trow[NMAX];
            t_factor_row<T, NMAX>(S.Sc, tau_sh, i, n, trow);
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
    pdl_begin();
    constexpr int B = NT * RPT;
    __shared__ FactorSmem<T, NMAX, NT, NORM64> S;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int64_t row0 = t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        factor_tile<T, NMAX, NT, RPT, NORM64>(S, p.M + row0, p.ld, ht, p.n, p.Rout + t * p.n, p.ldr);
    }
}

// ---------------------------------------------------------------------------
// Column-split tiles (n <= NMAX <= 64, tiles of 32*RPT rows, FP32 or FP64).
// The W = NMAX/CW warps of a CTA share one tile: warp w holds columns
// [w*CW, w*CW + CW) of all 32*RPT rows (row lane + 32*i in y[i]), so a
// thread carries RPT*CW tile values instead of RPT*NMAX and more rows fit on
// an SM.  Column j is owned by warp j/CW.  At step j the owner forms v_j and
// tau_j from its column, publishes them to shared memory and passes one CTA
// barrier; then every warp applies H_j to its own columns (dot products, a
// per-warp transpose reduction, the rank-1 update) while the owner goes on to
// column j+1.  Warps whose columns are all finished only take the dot
// products that give column j of V^T V.  The critical path of a step is the
// owner's chain for one CW-column block instead of the whole tile.  v_j
// alternates between two buffers: the owner rewrites buffer b at step j+2,
// after every warp has passed the barrier of step j+1 and so has read step
// j's copy.
//
// Every warp executes the same number of barriers (one per step; a phase of
// nloc columns runs 4*ceil(nloc/4) steps, the padding steps act on zero
// columns with tau = 0).  Output format as factor_tile.

__device__ __forceinline__ float fmadd(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }

// Reflector scalars on the owner's critical chain, FP32, branch-free: the
// hardware approximations refined by a Newton-Raphson step and finished with
// one residual correction each (Markstein's method for sqrt and reciprocal).  sqrt: r ~ 1/sqrt(x), r <- r (3 - x r^2) / 2,
// s = x r, s <- s + (r/2)(x - s^2) with the residual by FMA; reciprocal:
// r <- r (2 - x r), r <- r + r (1 - x r).  Both land within rounding of the
// correctly rounded results without the slow-path branches of the IEEE
// sequences.  Only used for x > 0 (the zero-column case selects other
// values).  FP64 keeps the exact operations.
__device__ __forceinline__ float refl_sqrt(float x) {
    float r = rsqrtf(x);
    r = r * fmaf(-0.5f * x * r, r, 1.5f);
    const float s = x * r;
    return fmaf(0.5f * r, fmaf(-s, s, x), s);
}
__device__ __forceinline__ double refl_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float refl_recip(float x) {
    float r = __fdividef(1.0f, x);
    r = r * fmaf(-x, r, 2.0f);
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}
__device__ __forceinline__ double refl_recip(double x) { return 1.0 / x; }

// 16-byte vector of T.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    static constexpr int N = 4;
    __device__ __forceinline__ static void store(float* p, const float* v) { *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]); }
    __device__ __forceinline__ static void load(const float* p, float* v) {
        const float4 q = *reinterpret_cast<const float4*>(p);
        v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
    }
};
template <>
struct Vec16<double> {
    static constexpr int N = 2;
    __device__ __forceinline__ static void store(double* p, const double* v) { *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]); }
    __device__ __forceinline__ static void load(const double* p, double* v) {
        const double2 q = *reinterpret_cast<const double2*>(p);
        v[0] = q.x, v[1] = q.y;
    }
};

// Row stride (elements) of the per-warp transpose scratch.  FP32 with CW = 4
// needs no padding (lane l's 16-byte row is words 4l..4l+3, and the column
// reads of the 8 lanes per position hit 32 distinct banks); other shapes
// get 16 bytes of pad.
template <typename T, int CW>
__host__ __device__ constexpr int colsum_stride() {
    return (sizeof(T) == 4 && CW == 4) ? 4 : CW + 16 / (int)sizeof(T);
}

// Layout of the published reflector: lane-major in 16-byte chunks when RPT
// allows (KC = RPT / VN chunks per lane, a power of two up to 8), so a lane moves its
// RPT values with KC vector accesses; chunk k of lane l sits at chunk
// position k ^ ((l / (8 / KC)) & (KC - 1)) of the lane's row, which puts the
// 8 lanes of each 16-byte access phase on 8 distinct 4-bank groups.
// Otherwise, or when VEC is false, slot i of lane l is element l + 32 i
// (scalar accesses).
template <typename T, int RPT, bool VEC = true>
struct VbufLayout {
    static constexpr int VN = Vec16<T>::N;
    static constexpr int KC = RPT / VN;
    static constexpr bool kVec = VEC && (RPT % VN == 0) && KC >= 1 && KC <= 8 && (KC & (KC - 1)) == 0;
    __device__ __forceinline__ static int swz(int lane) { return kVec ? (lane / (8 / KC)) & (KC - 1) : 0; }
    template <typename F>
    __device__ __forceinline__ static void store(T* buf, int lane, int sw, F&& val) {
        if constexpr (kVec) {
#pragma unroll
            for (int k = 0; k < KC; ++k) {
                T t[VN];
#pragma unroll
                for (int e = 0; e < VN; ++e) t[e] = val(k * VN + e);
                Vec16<T>::store(buf + lane * RPT + VN * (k ^ sw), t);
            }
        } else {
#pragma unroll
            for (int i = 0; i < RPT; ++i) buf[lane + 32 * i] = val(i);
        }
    }
    __device__ __forceinline__ static void load(const T* buf, int lane, int sw, T (&v)[RPT]) {
        if constexpr (kVec) {
#pragma unroll
            for (int k = 0; k < KC; ++k) Vec16<T>::load(buf + lane * RPT + VN * (k ^ sw), &v[k * VN]);
        } else {
#pragma unroll
            for (int i = 0; i < RPT; ++i) v[i] = buf[lane + 32 * i];
        }
    }
};

template <typename T, int NMAX, int CW, int RPT>
struct SplitFactorSmem {
    static constexpr int W = NMAX / CW;
    __align__(16) T vbuf[2][32 * RPT];
    T taub[2];
    __align__(16) T xpose[W][32 * colsum_stride<T, CW>()];
    __align__(16) T coef[W][CW];
    SCols<T, NMAX> Sc;
    T tau[NMAX];
    T rdiag[NMAX];
};

// CTA barrier 1 over `count` threads; non-aligned form, since the owner and
// the other warps reach it from different code.
__device__ __forceinline__ void step_barrier(int count) {
    asm volatile("barrier.sync 1, %0;\n" ::"r"(count) : "memory");
}

// Sum CW per-lane partials over the warp through a shared-memory transpose:
// returns, in lane l, the full sum of position l % CW (32/CW lanes hold each
// sum, bitwise equal).
template <typename T, int CW>
__device__ __forceinline__ T warp_colsum(const T (&q)[CW], T* scratch, int lane) {
    constexpr int SP = colsum_stride<T, CW>();
    constexpr int VN = Vec16<T>::N;
    constexpr int LPP = 32 / CW;  // lanes per position
    constexpr int RPL = 32 / LPP;  // rows summed by one lane
    T* mine = scratch + lane * SP;
#pragma unroll
    for (int c = 0; c < CW; c += VN) Vec16<T>::store(mine + c, &q[c]);
    __syncwarp();
    const int p = lane % CW, h = lane / CW;
    T a[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r) a[r] = scratch[(h + LPP * r) * SP + p];
#pragma unroll
    for (int w = RPL / 2; w >= 1; w >>= 1)
#pragma unroll
        for (int r = 0; r < w; ++r) a[r] += a[r + w];
    T s = a[0];
#pragma unroll
    for (int o = CW; o < 32; o <<= 1) s += __shfl_xor_sync(kFull, s, o);
    __syncwarp();  // scratch is rewritten by the next call
    return s;
}

// VECV: publish the reflector in the 16-byte vector layout (VbufLayout).
// Off for the 64-column tile and for the batched kernels, whose registers
// leave no room for the aligned quads it needs (more spills with it).
// N64: the owner's column norm (sigma^2, accumulated and reduced), alpha and
// the reflector scalars beta, tau and 1/(alpha - beta) in FP64, rounded to
// the tile's type once computed; the tile, the dot products and the updates
// stay in T.  (The precision form's option fp64_scalars.)
// The tile comes from global memory (Hook = NoHook), or from a copy in
// shared memory staged by TMA (any other Hook; stile): 256-row boxes of
// NMAX columns, box h holding rows [256h, 256h + 256) column by column, the
// rows past the level's end and the columns past n already zero.  `loaded`
// runs once every thread holds its values.
struct NoHook {
    __device__ __forceinline__ void operator()() const {}
};
template <typename T, int NMAX, int CW, int RPT, bool VECV = (NMAX <= 32), bool N64 = false, class Hook = NoHook>
__device__ __forceinline__ void factor_split_tile(SplitFactorSmem<T, NMAX, CW, RPT>& S, T* tile, int64_t ld, int ht,
                                                  int n, T* Rt, int64_t ldr, const T* stile = nullptr,
                                                  Hook loaded = Hook()) {
    using SC = typename std::conditional<N64, double, T>::type;  // type of the reflector scalars
    constexpr int W = NMAX / CW;
    constexpr int U = 4;
    constexpr int VN = Vec16<T>::N;
    static_assert(NMAX <= 64 && CW % U == 0 && CW % VN == 0 && NMAX % CW == 0 && W >= 2 && 32 * RPT >= NMAX &&
                      W >= NMAX / 32,
                  "bad split configuration");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int col0 = warp * CW;
    const int mycols = max(0, min(CW, n - col0));
    T* scratch = S.xpose[warp];
    using VL = VbufLayout<T, RPT, VECV>;
    const int vsw = VL::swz(lane);
    // Row lane + 32*i lies strictly below diagonal element j (compile-time
    // true for every slot i >= 1 when NMAX <= 32).
    auto below = [&](int i, int j) { return (NMAX <= 32 && i > 0) || (lane + 32 * i > j); };
    // Reflector scalars: the branch-free forms shorten the owner's chain for
    // NMAX <= 32; the 64-column tile, already at its register limit, runs
    // faster with the plain operations (level-0 factor at 4,194,304 x 64:
    // 3.25 against 3.78 ms).
    auto rsq = [](SC x) {
        if constexpr (NMAX <= 32) return refl_sqrt(x);
        else return sqrt_t(x);
    };
    auto rcp = [](SC x) {
        if constexpr (NMAX <= 32) return refl_recip(x);
        else return recip(x);
    };
    // x(j, c) of position c, held by lane j % 32 in slot j / 32 (j < 64)
    auto diag_slot = [&](const T(&yy)[RPT][CW], int c, int j) {
        return (NMAX > 32 && j >= 32) ? yy[RPT > 1 ? 1 : 0][c] : yy[0][c];
    };

    T y[RPT][CW];
    if constexpr (!std::is_same<Hook, NoHook>::value) {
        // rows lane + 32 i of box i / 8, consecutive lanes on consecutive words
        const T* s0 = stile + col0 * 256 + lane;
#pragma unroll
        for (int c = 0; c < CW; ++c)
#pragma unroll
            for (int i = 0; i < RPT; ++i) y[i][c] = s0[((i >> 3) * NMAX + c) * 256 + 32 * (i & 7)];
    } else {
        // one column pointer stepped by ld; the row offsets 32*i are immediates
        const T* pcol = tile + (int64_t)col0 * ld + lane;
#pragma unroll
        for (int c = 0; c < CW; ++c) {
#pragma unroll
            for (int i = 0; i < RPT; ++i) y[i][c] = (lane + 32 * i < ht && c < mycols) ? pcol[32 * i] : T(0);
            pcol += ld;
        }
    }
    loaded();
    int shift = 0;  // after this warp's own phase, position c holds its local column (c + shift) % CW

#pragma unroll 1
    for (int ph = 0; ph < W; ++ph) {
        const int pc0 = ph * CW;
        const int nloc = min(CW, n - pc0);
        if (nloc <= 0) break;  // same for every warp
        const int G = (nloc + U - 1) / U;
        if (warp == ph) {
            // ---- owner: reflectors of columns pc0 .. pc0+nloc-1, in groups of
            // U with the register rotation of factor_tile, and the norm of the
            // next column reduced while the current update is issued
            SC sig2, alpha;
            {
                SC s4[4] = {SC(0), SC(0), SC(0), SC(0)};
#pragma unroll
                for (int i = 0; i < RPT; ++i)
                    if (below(i, pc0)) s4[i & 3] = fmadd((SC)y[i][0], (SC)y[i][0], s4[i & 3]);
                alpha = (SC)__shfl_sync(kFull, diag_slot(y, 0, pc0), pc0 & 31);
                sig2 = warp_sum((s4[0] + s4[1]) + (s4[2] + s4[3]));
            }
#pragma unroll 1
            for (int g = 0; g < G; ++g) {
                const int base = U * g;
                const int live = nloc - base;
                const int past0 = CW - base;
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = pc0 + base + u;
                    const bool zero = (sig2 == SC(0));
                    const SC nrm = rsq(fmadd(alpha, alpha, sig2));
                    const SC beta_s = zero ? alpha : ((alpha >= SC(0)) ? -nrm : nrm);
                    const T beta = (T)beta_s;
                    const T tau = zero ? T(0) : (T)((beta_s - alpha) * rcp(beta_s));
                    const T scale = zero ? T(0) : (T)rcp(alpha - beta_s);
#pragma unroll
                    for (int i = 0; i < RPT; ++i)
                        if (below(i, j)) y[i][u] *= scale;
                    // v_j of slot i (1 on the diagonal, 0 above it)
                    auto vj = [&](int i) { return below(i, j) ? y[i][u] : ((lane + 32 * i == j) ? T(1) : T(0)); };
                    const int b = j & 1;
                    VL::store(S.vbuf[b], lane, vsw, vj);
                    if (lane == 0) {
                        S.taub[b] = tau;
                        S.tau[j] = tau;
                        S.rdiag[j] = beta;
                    }
                    step_barrier(W * 32);
                    T q[CW];
#pragma unroll
                    for (int c = 0; c < CW; ++c) {
                        q[c] = (c != u) ? vj(0) * y[0][c] : T(0);
#pragma unroll
                        for (int i = 1; i < RPT; ++i)
                            if (c != u) q[c] = fmadd(vj(i), y[i][c], q[c]);
                    }
                    const T d = warp_colsum<T, CW>(q, scratch, lane);
                    if (lane < CW) {
                        S.coef[warp][lane] = (lane > u && lane < live) ? d : T(0);
                        const int k = (lane >= past0) ? lane - past0 : ((lane < u) ? base + lane : -1);
                        if (k >= 0) S.Sc.c[j][pc0 + k] = d;
                    }
                    __syncwarp();
                    T tv[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) tv[i] = tau * vj(i);
                    T cf[CW];
#pragma unroll
                    for (int c0 = 0; c0 < CW; c0 += VN) {
                        if (c0 + VN - 1 <= u) continue;
                        Vec16<T>::load(&S.coef[warp][c0], &cf[c0]);
                    }
                    if (u + 1 < CW) {
                        const int c = (u + 1 < CW) ? u + 1 : 0;  // keeps the index in range when u + 1 == CW
#pragma unroll
                        for (int i = 0; i < RPT; ++i) y[i][c] = fmadd(-tv[i], cf[c], y[i][c]);
                        SC s4[4] = {SC(0), SC(0), SC(0), SC(0)};  // four chains instead of one RPT-deep one
#pragma unroll
                        for (int i = 0; i < RPT; ++i)
                            if (below(i, j + 1)) s4[i & 3] = fmadd((SC)y[i][c], (SC)y[i][c], s4[i & 3]);
                        alpha = (SC)__shfl_sync(kFull, diag_slot(y, c, j + 1), (j + 1) & 31);
                        sig2 = warp_sum((s4[0] + s4[1]) + (s4[2] + s4[3]));
                    }
#pragma unroll
                    for (int c = u + 2; c < CW; ++c)
#pragma unroll
                        for (int i = 0; i < RPT; ++i) y[i][c] = fmadd(-tv[i], cf[c], y[i][c]);
                }
#pragma unroll
                for (int i = 0; i < RPT; ++i) {
                    T keep[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) keep[u] = y[i][u];
#pragma unroll
                    for (int c = 0; c < CW - U; ++c) y[i][c] = y[i][c + U];
#pragma unroll
                    for (int u = 0; u < U; ++u) y[i][CW - U + u] = keep[u];
                }
            }
            shift = (U * G) % CW;
        } else {
            // ---- the other warps: apply H_j (later columns) or take column j
            // of V^T V (finished columns), one barrier per step as the owner
            const bool trailing = warp > ph;
#pragma unroll 1
            for (int st = 0; st < G * U; ++st) {
                const int j = pc0 + st;
                step_barrier(W * 32);
                const int b = j & 1;
                T v[RPT];
                VL::load(S.vbuf[b], lane, vsw, v);
                const T tau = S.taub[b];
                T q[CW];
#pragma unroll
                for (int c = 0; c < CW; ++c) {
                    q[c] = v[0] * y[0][c];
#pragma unroll
                    for (int i = 1; i < RPT; ++i) q[c] = fmadd(v[i], y[i][c], q[c]);
                }
                const T d = warp_colsum<T, CW>(q, scratch, lane);
                if (trailing) {
                    if (lane < CW) S.coef[warp][lane] = d;
                    __syncwarp();
                    T tv[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) tv[i] = tau * v[i];
#pragma unroll
                    for (int c0 = 0; c0 < CW; c0 += VN) {
                        T w[VN];
                        Vec16<T>::load(&S.coef[warp][c0], w);
#pragma unroll
                        for (int e = 0; e < VN; ++e)
#pragma unroll
                            for (int i = 0; i < RPT; ++i) y[i][c0 + e] = fmadd(-tv[i], w[e], y[i][c0 + e]);
                    }
                } else if (lane < CW) {
                    const int kl = (lane + shift) % CW;
                    if (kl < mycols) S.Sc.c[j][col0 + kl] = d;
                }
            }
        }
    }
    step_barrier(W * 32);  // tau, rdiag and V^T V complete

    // R (row r < n sits in slot r / 32 of lane r % 32 in the warp holding
    // column k) and V below the diagonal, each warp for its own columns.
#pragma unroll
    for (int c = 0; c < CW; ++c) {
        const int kl = (c + shift) % CW;
        if (kl < mycols) {
            const int k = col0 + kl;
#pragma unroll
            for (int i = 0; i < (NMAX + 31) / 32; ++i) {
                const int r = lane + 32 * i;
                if (r < n) {
                    T v = (k > r) ? y[i][c] : ((k == r) ? S.rdiag[r] : T(0));
                    if (r >= ht) v = T(0);
                    Rt[r + (int64_t)k * ldr] = v;
                }
            }
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int r = lane + 32 * i;
                if (r < ht && r > k) tile[r + (int64_t)k * ld] = y[i][c];
            }
        }
    }
    // T in the top block's upper triangle (diagonal included), row i by
    // thread i: T(i,i) = tau_i, T(i,j) = -tau_j sum_{k=i}^{j-1} T(i,k) S(k,j).
    {
        const int i = threadIdx.x;
        if (i < n && i < ht) {
            T trow[NMAX];
            t_factor_row<T, NMAX>(S.Sc, S.tau, i, n, trow);
#pragma unroll
            for (int j = 0; j < NMAX; ++j)
                if (j >= i && j < n) tile[i + (int64_t)j * ld] = trow[j];
        }
    }
    step_barrier(W * 32);  // S is reused by the CTA's next tile
}

template <typename T, int NMAX, int CW, int RPT, int MINB, bool N64 = false>
__global__ void __launch_bounds__(32 * (NMAX / CW), MINB) factor_split_tiles(FactorParams<T> p) {
    pdl_begin();
    constexpr int B = 32 * RPT;
    __shared__ SplitFactorSmem<T, NMAX, CW, RPT> S;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int64_t row0 = t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        factor_split_tile<T, NMAX, CW, RPT, (NMAX <= 32), N64>(S, p.M + row0, p.ld, ht, p.n, p.Rout + t * p.n, p.ldr);
    }
}

// Persistent form of factor_split_tiles whose tiles are staged into shared
// memory by TMA (two 256-row boxes of a 512-row tile, rows past the level's
// end filled with zeros by the copy itself): a CTA waits for its tile, every
// thread takes its values into registers, and the TMA of the CTA's next tile
// is issued while the current one is factored, so the tile load leaves the
// tile's chain.  The wait is bounded: after p.tries polls the CTA sets the
// status word, waits (with the full limit) for the copy in flight and stops.
// Dynamic shared memory of the TMA form: the tile's boxes, then the
// mbarrier that counts their bytes (both at fixed offsets, so neither
// address takes a register across the tile).
extern __shared__ __align__(128) unsigned char tma_stage[];
template <typename T, int NMAX, int CW, int RPT>
constexpr size_t tma_tile_bytes() {
    return (size_t)(RPT / 8) * NMAX * 256 * sizeof(T);
}
template <typename T, int NMAX, int CW, int RPT>
constexpr size_t tma_stage_bytes() {
    return tma_tile_bytes<T, NMAX, CW, RPT>() + 16;
}
// One thread: the copies of the tile whose first row is y, counted on the
// stage's mbarrier.
template <int BOXES, int BOX_BYTES>
__device__ __forceinline__ void tma_issue_tile(const CUtensorMap* tmap, int y) {
    const uint32_t dst = tc::smem_u32(tma_stage), mb = dst + BOXES * BOX_BYTES;
    tc::fence_smem_to_async();
    tc::mbar_arrive_expect_tx(mb, (uint32_t)(BOXES * BOX_BYTES));
#pragma unroll
    for (int h = 0; h < BOXES; ++h) tc::tma_load_2d(dst + h * BOX_BYTES, tmap, y + h * 256, 0, mb);
}
// The `loaded` hook of the TMA form: every thread holds its values, so the
// buffer is free and thread 0 (go) starts the next tile's copy.  Held by
// value: a hook that referred to the loop's locals would put them on the
// stack.
template <int BOXES, int BOX_BYTES>
struct TmaNextTile {
    const CUtensorMap* tmap;
    int y;
    bool go;
    __device__ __forceinline__ void operator()() const {
        __syncthreads();
        if (go) tma_issue_tile<BOXES, BOX_BYTES>(tmap, y);
    }
};
template <typename T, int NMAX, int CW, int RPT, int MINB>
__global__ void __launch_bounds__(32 * (NMAX / CW), MINB)
    factor_split_tiles_tma(FactorParams<T> p, const __grid_constant__ CUtensorMap tmap) {
    pdl_begin();
    static_assert(RPT % 8 == 0, "tiles of whole 256-row boxes");
    constexpr int B = 32 * RPT, BOXES = RPT / 8, BOX_BYTES = NMAX * 256 * (int)sizeof(T);
    __shared__ SplitFactorSmem<T, NMAX, CW, RPT> S;
    const T* stile = reinterpret_cast<const T*>(tma_stage);
    const uint32_t mb = tc::smem_u32(tma_stage) + BOXES * BOX_BYTES;
    if (threadIdx.x == 0) {
        tc::mbar_init(mb, 1);
        tc::fence_mbar_init();
    }
    __syncthreads();
    // Row coordinates fit 32 bits (TMA takes them signed; the host launches
    // this kernel for ntiles * B <= INT32_MAX only).  The loop carries one
    // counter k (tile
    // blockIdx.x + k gridDim.x, mbarrier phase k & 1) across the tile's
    // body, which needs every register it can get.
    const int ntiles = (int)p.ntiles;
    if (threadIdx.x == 0 && (int)blockIdx.x < ntiles)
        tma_issue_tile<BOXES, BOX_BYTES>(&tmap, (int)blockIdx.x * B);
#pragma unroll 1
    for (int k = 0;; ++k) {
        const int t = (int)blockIdx.x + k * (int)gridDim.x;
        if (t >= (int)p.ntiles) break;
        const uint32_t phase = (uint32_t)k & 1u;
        const bool ok = tc::mbar_wait(mb, phase, p.tries);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) {
                if (p.err) atomicExch(p.err, 1);
                // the copy in flight must not land after the CTA is gone:
                // this wait keeps the full limit
                (void)tc::mbar_wait(mb, phase);
            }
            break;
        }
        const int64_t row0 = (int64_t)t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        const int tn = t + (int)gridDim.x;
        const TmaNextTile<BOXES, BOX_BYTES> loaded{&tmap, tn * B, threadIdx.x == 0 && tn < (int)p.ntiles};
        factor_split_tile<T, NMAX, CW, RPT, (NMAX <= 32), false>(S, p.M + row0, p.ld, ht, p.n, p.Rout + t * p.n,
                                                                  p.ldr, stile, loaded);
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

        {
            // all global reads first: interleaved with the shared stores they
            // would be issued one at a time (the generic pointers may alias)
            constexpr int PER = (NMAX * NMAX + NT - 1) / NT;
            T tv[PER], bv[PER];
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                const int idx = tid + NT * e;
                const int r = idx % NMAX, c = idx / NMAX;
                const bool ok = idx < NMAX * NMAX;
                tv[e] = (ok && r < ht && r < n && c < n) ? tile[r + c * p.ld] : T(0);
                if (p.P)
                    bv[e] = (ok && r < n && c < n) ? p.P[t * n + r + c * p.ldp] : T(0);
                else
                    bv[e] = (r == c && r < n) ? T(1) : T(0);
            }
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                const int idx = tid + NT * e;
                const int r = idx % NMAX, c = idx / NMAX;
                if (idx < NMAX * NMAX) {
                    Vt[r][c] = (r > c) ? tv[e] : ((r == c && c < n) ? T(1) : T(0));
                    Tt[r][c] = (r <= c) ? tv[e] : T(0);
                    Bs[r][c] = bv[e];
                }
            }
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
        if constexpr (std::is_same<T, float>::value && NMAX % 4 == 0) {
            // FP32: each row's accumulators as column pairs, updated with the
            // packed FP32x2 FMA (each half rounded as fmaf): a 16-byte read
            // of W's row k gives two pairs, and only the row's V value is
            // duplicated -- about 40% fewer instructions in this
            // issue-bound loop.
            float2 q[RPT][NMAX / 2];
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int r = tid + NT * i;
#pragma unroll
                for (int c = 0; c < NMAX; c += 2)
                    q[i][c / 2] = (r < n) ? make_float2(Bs[r][c], Bs[r][c + 1]) : make_float2(0.f, 0.f);
            }
#pragma unroll 8
            for (int k = 0; k < NMAX; ++k) {
                if (k < n) {
                    float2 nv[RPT];
#pragma unroll
                    for (int i = 0; i < RPT; ++i) {
                        const int r = tid + NT * i;
                        const float v = (r < n) ? Vt[r][k] : ((r < ht) ? Vs[(size_t)k * B + r] : 0.f);
                        nv[i] = make_float2(-v, -v);
                    }
#pragma unroll
                    for (int c0 = 0; c0 < NMAX; c0 += 4) {
                        const float4 w = *reinterpret_cast<const float4*>(&Ws[k][c0]);
#pragma unroll
                        for (int i = 0; i < RPT; ++i) {
                            q[i][c0 / 2] = __ffma2_rn(nv[i], make_float2(w.x, w.y), q[i][c0 / 2]);
                            q[i][c0 / 2 + 1] = __ffma2_rn(nv[i], make_float2(w.z, w.w), q[i][c0 / 2 + 1]);
                        }
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const int r = tid + NT * i;
                if (r < ht) {
#pragma unroll
                    for (int c = 0; c < NMAX; ++c)
                        if (c < n) tile[r + c * p.ld] = (c & 1) ? q[i][c / 2].y : q[i][c / 2].x;
                }
            }
        } else {
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
        }
        __syncthreads();
    }
}

template <typename T, int NMAX, int NT, int RPT, int MINB>
__global__ void __launch_bounds__(NT, MINB) apply_tiles(ApplyParams<T> p) {
    pdl_begin();
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
