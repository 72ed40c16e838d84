// tc_apply.cu -- Q assembly of the TSQR down-sweep on the tcgen05 tensor
// cores (precision form, FP32 entry points).
//
// Same arithmetic as apply_tiles (the down-sweep of kernelQR.h:397-492 and
// tsgemm_tsqr, TallShinnyQR.h:11-74): for each tile, Q = [B;0] - V W with
// W = T (V_top^T B).  The small n x n products that give W stay on CUDA
// cores in FP32.  The bulk product V W (tile rows x n x n) runs as
// tcgen05.mma kind::tf32 with FP32 accumulation in TMEM, with both operands
// split into TF32 hi + lo parts and three products hi*hi + hi*lo + lo*hi, so
// the result carries close to FP32 accuracy (about 2^-21 relative per
// product).
//
// One CTA of 128 threads (one warpgroup) takes a tile and walks it in blocks
// of 128 rows: each thread loads its row of V (coalesced column loads),
// splits it and stores both halves as the K-major A operand; one thread
// issues 3 * NMAX/8 MMAs (M = 128, N = NMAX, K = 8) and commits them to an
// mbarrier; each warp then reads its 32 TMEM lanes (its 32 rows) and writes
// Q.  The next block's row is loaded into registers before the wait, so the
// global loads overlap the tensor-core work.  The B operand holds -W, so the
// MMA result D = -V W is Q itself below the tile's top n rows (Q = B + D
// there), and a level with n = NMAX takes an instantiation without column
// tests: at 4,194,304 x 32 level 0 went from 0.301 to 0.266 ms.
#include <cuda_runtime.h>

#include "internal.h"
#include "tc.cuh"
#include "tsqr_kernels.cuh"

namespace tsqr {

namespace {

template <int NMAX>
struct TcApplySmem {
    uint32_t b_hi[NMAX * NMAX];    // K-major B operand: W (K = NMAX rows of W, N = NMAX)
    uint32_t b_lo[NMAX * NMAX];
    float Vt[NMAX][NMAX + 1];      // masked top block of V (read again by block 0)
    // the parent block B (read again by the epilogue); rows padded to 16
    // bytes so the W products read a row's columns as vectors
    __align__(16) float Bs[NMAX][NMAX + 4];
    union {
        struct {                   // K-major A operand, one 128-row block
            uint32_t a_hi[128 * NMAX];
            uint32_t a_lo[128 * NMAX];
        } op;
        struct {                   // scratch of the W products, dead before staging starts
            float Tt[NMAX][NMAX + 1];
            __align__(16) float Ys[NMAX][NMAX + 4];
        } w;
    } u;
    unsigned long long mbar;
    uint32_t tmem_slot;
};

// NF: n == NMAX (no column tests).  Threads: 128 for NMAX <= 32 (4 CTAs
// per SM); 256 for NMAX = 64 (one CTA per SM, whose shared memory is
// 130 KB): there thread t owns row t % 128 of each block and columns
// 32 (t / 128) .. +31, so its rows, prefetch and TMEM read stay at 32
// values; warp w reads TMEM lanes 32 (w % 4) .. +31 of its column half.
template <int NMAX>
constexpr int tc_apply_threads() {
    return NMAX <= 32 ? 128 : 256;
}
template <int NMAX, int B, bool NF>
__global__ void __launch_bounds__(tc_apply_threads<NMAX>(), NMAX <= 32 ? 4 : 1)
    tc_apply_tiles(ApplyParams<float> p, int* err, int tries) {
    pdl_begin();
    static_assert(NMAX % 16 == 0 && NMAX <= 64 && B % 128 == 0, "bad shape");
    constexpr int NT = tc_apply_threads<NMAX>();
    constexpr int HC = NMAX * 128 / NT;  // columns a thread owns in the block phase
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    TcApplySmem<NMAX>& S = *reinterpret_cast<TcApplySmem<NMAX>*>(tc_smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int rb = tid & 127, cb = (tid >> 7) * HC;  // row in the block, first column
    const int n = p.n;
    constexpr uint32_t kCols = NMAX < 32 ? 32 : NMAX;  // TMEM columns: power of 2 >= 32
    constexpr uint32_t idesc = tc::idesc_tf32(128, NMAX);
    constexpr uint32_t SBO = NMAX * 32;  // bytes between 8-row groups of a K-major tile with K = NMAX

    const uint32_t mbar = tc::smem_u32(&S.mbar);
    if (warp == 0) tc::tmem_alloc(&S.tmem_slot, kCols);
    if (tid == 0) {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem_slot;
    uint32_t phase = 0;
    bool ok = true;

    // Row `blk*128 + rb`, columns cb.., of tile tt into v (zero past the tile; the top
    // n rows come masked from Vt instead).  Issued one block ahead, and for
    // the first block of the next tile before this tile's W products, so
    // the global loads are in flight while the CTA computes.
    float vnext[HC];
    auto load_block = [&](int64_t tt, int blk, float(&v)[HC]) {
        const int64_t r0 = tt * B;
        const int htt = (int)((p.h - r0) < B ? (p.h - r0) : B);
        const float* tl = p.M + r0;
        const int r = blk * 128 + rb;
        const bool rok = r >= n && r < htt;  // the top n rows come from Vt
#pragma unroll
        for (int j = 0; j < HC; ++j)
            v[j] = (rok && (NF || cb + j < n)) ? tl[r + (int64_t)(cb + j) * p.ld] : 0.f;
    };
    if (blockIdx.x < p.ntiles) load_block(blockIdx.x, 0, vnext);

    for (int64_t t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
        const int64_t row0 = t * B;
        const int ht = (int)((p.h - row0) < B ? (p.h - row0) : B);
        float* tile = p.M + row0;

        // --- W = T (V_top^T B) on CUDA cores, then W as the B operand -----
        {
            // all global reads first: interleaved with the shared stores they
            // would be issued one at a time (the generic pointers may alias)
            constexpr int PER = NMAX * NMAX / NT;
            float tv[PER], bv[PER];
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                const int idx = tid + NT * e;
                const int r = idx % NMAX, c = idx / NMAX;
                tv[e] = (r < ht && r < n && c < n) ? tile[r + c * p.ld] : 0.f;
                if (p.P)
                    bv[e] = (r < n && c < n) ? p.P[t * n + r + c * p.ldp] : 0.f;
                else
                    bv[e] = (r == c && r < n) ? 1.f : 0.f;
            }
#pragma unroll
            for (int e = 0; e < PER; ++e) {
                const int idx = tid + NT * e;
                const int r = idx % NMAX, c = idx / NMAX;
                S.Vt[r][c] = (r > c) ? tv[e] : ((r == c && c < n) ? 1.f : 0.f);
                S.u.w.Tt[r][c] = (r <= c) ? tv[e] : 0.f;
                S.Bs[r][c] = bv[e];
            }
        }
        __syncthreads();
        // Each thread owns output row k and the CPT contiguous columns
        // c0 .. c0+CPT-1: per term one shared load of its own operand and
        // CPT/4 16-byte loads of the other, which every lane of the warp
        // reads at the same address (broadcast).
        constexpr int CPT = NMAX * NMAX / NT;
        static_assert(CPT % 2 == 0 && CPT <= 16, "W products read 8- or 16-byte groups");
        const int k = tid % NMAX, c0 = (tid / NMAX) * CPT;
        auto row_terms = [&](const float* row, float(&a)[CPT], float x) {
            if constexpr (CPT % 4 == 0) {
#pragma unroll
                for (int j = 0; j < CPT; j += 4) {
                    const float4 q = *reinterpret_cast<const float4*>(row + c0 + j);
                    a[j] = fmaf(x, q.x, a[j]);
                    a[j + 1] = fmaf(x, q.y, a[j + 1]);
                    a[j + 2] = fmaf(x, q.z, a[j + 2]);
                    a[j + 3] = fmaf(x, q.w, a[j + 3]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < CPT; j += 2) {
                    const float2 q = *reinterpret_cast<const float2*>(row + c0 + j);
                    a[j] = fmaf(x, q.x, a[j]);
                    a[j + 1] = fmaf(x, q.y, a[j + 1]);
                }
            }
        };
        {
            float acc[CPT];
#pragma unroll
            for (int j = 0; j < CPT; ++j) acc[j] = 0.f;
#pragma unroll
            for (int r = 0; r < NMAX; ++r) row_terms(S.Bs[r], acc, S.Vt[r][k]);
#pragma unroll
            for (int j = 0; j < CPT; ++j) S.u.w.Ys[k][c0 + j] = acc[j];  // Y = V_top^T B
        }
        __syncthreads();
        {
            float acc[CPT];
#pragma unroll
            for (int j = 0; j < CPT; ++j) acc[j] = 0.f;
#pragma unroll
            for (int l = 0; l < NMAX; ++l) row_terms(S.u.w.Ys[l], acc, S.u.w.Tt[k][l]);
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                // -W = -T Y as the B operand (row = output column c, K index
                // k): the MMA then gives D = -V W, which is Q itself below
                // the top block
                uint32_t hi, lo;
                tc::split_tf32(-acc[j], hi, lo);
                const uint32_t off = tc::kmajor_off(c0 + j, k, NMAX) >> 2;
                S.b_hi[off] = hi;
                S.b_lo[off] = lo;
            }
        }

        // --- blocks of 128 rows ------------------------------------------
        const int nblk = (ht + 127) / 128;
        __syncthreads();  // Vt complete (masked top rows)
        for (int blk = 0; blk < nblk; ++blk) {
            const int r = blk * 128 + rb;
            float v[HC];
#pragma unroll
            for (int j = 0; j < HC; ++j) v[j] = (r < n) ? S.Vt[r][cb + j] : vnext[j];
#pragma unroll
            for (int k4 = 0; k4 < HC; k4 += 4) {
                uint4 hi, lo;
                tc::split_tf32(v[k4 + 0], hi.x, lo.x);
                tc::split_tf32(v[k4 + 1], hi.y, lo.y);
                tc::split_tf32(v[k4 + 2], hi.z, lo.z);
                tc::split_tf32(v[k4 + 3], hi.w, lo.w);
                const uint32_t off = tc::kmajor_off(rb, cb + k4, NMAX);
                *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.u.op.a_hi) + off) = hi;
                *reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.u.op.a_lo) + off) = lo;
            }
            tc::fence_smem_to_async();
            tc::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc::fence_after_sync();
                const uint32_t ah = tc::smem_u32(S.u.op.a_hi), al = tc::smem_u32(S.u.op.a_lo);
                const uint32_t bh = tc::smem_u32(S.b_hi), bl = tc::smem_u32(S.b_lo);
#pragma unroll
                for (int ks = 0; ks < NMAX / 8; ++ks) {
                    const uint32_t ko = ks * 256;  // two core matrices of 16 bytes of K
                    const uint64_t dah = tc::smem_desc(ah + ko, 128, SBO), dal = tc::smem_desc(al + ko, 128, SBO);
                    const uint64_t dbh = tc::smem_desc(bh + ko, 128, SBO), dbl = tc::smem_desc(bl + ko, 128, SBO);
                    tc::mma_tf32(tmem, dah, dbh, idesc, ks > 0);
                    tc::mma_tf32(tmem, dah, dbl, idesc, true);
                    tc::mma_tf32(tmem, dal, dbh, idesc, true);
                }
                tc::mma_commit(mbar);
            }
            // prefetch the next block's rows while the tensor core works
            if (blk + 1 < nblk)
                load_block(t, blk + 1, vnext);
            else if (t + gridDim.x < p.ntiles)
                load_block(t + gridDim.x, 0, vnext);
            const bool waited = tc::mbar_wait(mbar, phase, tries);
            // a timed-out wait anywhere stops the whole CTA (uniform decision)
            if (__syncthreads_or(!waited)) {
                ok = false;
                if (tid == 0) atomicExch(err, 1);
                break;
            }
            phase ^= 1u;
            tc::fence_after_sync();
            // epilogue: warp w owns TMEM lanes 32 (w % 4) .. +31 = rows rb
            // of the block, columns cb .. cb + HC - 1
            float d[HC];
#pragma unroll
            for (int c8 = 0; c8 < HC; c8 += 8) {
                float d8[8];
                tc::tmem_ld8(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(cb + c8), d8);
#pragma unroll
                for (int e = 0; e < 8; ++e) d[c8 + e] = d8[e];
            }
            tc::tmem_ld_wait();
            if (r < ht) {
                if (r < n) {  // the top block: Q = B + D
#pragma unroll
                    for (int j = 0; j < HC; ++j)
                        if (NF || cb + j < n) tile[r + (int64_t)(cb + j) * p.ld] = S.Bs[r][cb + j] + d[j];
                } else {  // below it: Q = D
#pragma unroll
                    for (int j = 0; j < HC; ++j)
                        if (NF || cb + j < n) tile[r + (int64_t)(cb + j) * p.ld] = d[j];
                }
            }
            tc::fence_before_sync();
            __syncthreads();  // TMEM and the A buffers are free for the next block
        }
    }
    if (!ok) {
        // give the MMAs still in flight a bounded chance to retire before
        // the TMEM they write is released
        (void)tc::mbar_wait(mbar, phase);
    }
    tc::fence_after_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

template <int NMAX, int B>
void launch(const ApplyParams<float>& p, int grid, int* err, cudaStream_t s) {
    constexpr size_t smem = sizeof(TcApplySmem<NMAX>) + 1024;
    static PerDeviceOnce attr;
    attr.run([] {
        cudaFuncSetAttribute(tc_apply_tiles<NMAX, B, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(tc_apply_tiles<NMAX, B, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    const int tries = wait_tries().load(std::memory_order_relaxed);
    constexpr int NT = tc_apply_threads<NMAX>();
    if (p.n == NMAX)
        launch_pdl(tc_apply_tiles<NMAX, B, true>, dim3(grid), dim3(NT), smem, s, p, err, tries);
    else
        launch_pdl(tc_apply_tiles<NMAX, B, false>, dim3(grid), dim3(NT), smem, s, p, err, tries);
}

}  // namespace

// Tile heights must match the factor configuration of the precision path.
bool tc_apply_level(const ApplyParams<float>& p, int nmax, int rows, int* err, cudaStream_t s) {
    // persistent grid: resident CTAs walk the tiles, prefetching the next one
    const int sms = device_sm_count();
    const int64_t resident = (int64_t)sms * (nmax <= 32 ? 4 : 1);
    const int grid = (int)(p.ntiles < 1 ? 1 : (p.ntiles > resident ? resident : p.ntiles));
    if (nmax == 64 && rows == 512) {
        launch<64, 512>(p, grid, err, s);
    } else if (nmax == 32 && rows == 512) {
        launch<32, 512>(p, grid, err, s);
    } else if (nmax == 16 && rows == 512) {
        launch<16, 512>(p, grid, err, s);
    } else {
        return false;
    }
    return true;
}

}  // namespace tsqr
