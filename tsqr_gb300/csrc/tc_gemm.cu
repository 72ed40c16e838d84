// tc_gemm.cu -- the blocked-QR trailing GEMMs on the tcgen05 tensor cores
// (precision form of qr<float>, block_QR.h:72-95).
//
// The reference's naive gemm_blockqr (block_QR.h:7-60) computes
//   R12 = A1^T A2      (op = T, a length-m dot per thread) and
//   A2  = A2 - A1 R12  (op = N).
// Here both run as tcgen05.mma kind::tf32 with FP32 accumulation in TMEM and
// the operands split into TF32 hi + lo (three products hi*hi + hi*lo +
// lo*hi, about 2^-21 relative per product).
//
// tc_gemm_kernel<TRANS_A>: a CTA of 128 threads owns a 128 x NB block of the
// output (TMEM lanes = output rows, NB fp32 columns) and walks its K range
// in stages of 32.  Per stage every thread loads its share of the A and B
// slices, splits them and stores the K-major operand tiles; one thread
// issues 3 x 4 MMAs (M = 128, N = NB, K = 8) and commits them to the stage's
// mbarrier.  Two stage buffers alternate, so the loads of stage s+1 overlap
// the MMAs of stage s.
//   TRANS_A = true : D = A^T B over rows [k0, k1) of A (K x M) and B (K x N)
//                    -> written as a partial sum P_z (M x N), summed later
//                    (deterministic split-K, no atomics).
//   TRANS_A = false: D = A B with A (M x K) and B (K x N) small
//                    -> C = C + alpha * D.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "tc.cuh"

namespace tsqr {

namespace {

constexpr int KS = 32;  // K per stage

template <int NB>
struct GemmSmem {
    uint32_t a_hi[2][128 * KS];
    uint32_t a_lo[2][128 * KS];
    uint32_t b_hi[2][NB * KS];
    uint32_t b_lo[2][NB * KS];
    unsigned long long mbar[2];
    uint32_t tmem_slot;
};

// BF: BF16x3 instead of TF32x3 -- the same K-major tiles hold 16-bit
// values (a core matrix row = 8 values of K), and each MMA (kind::f16, both
// operands BF16) covers K = 16.
template <bool TRANS_A, int NB, bool BF = false>
__global__ void __launch_bounds__(128) tc_gemm_kernel(int M, int N, int64_t K, const float* __restrict__ A, int64_t lda,
                                                      const float* __restrict__ Bm, int64_t ldb, float* __restrict__ C,
                                                      int64_t ldc,
                                                      float alpha, int64_t kchunk, int* err, int tries) {
    pdl_begin();
    extern __shared__ __align__(1024) unsigned char gemm_smem_raw[];
    GemmSmem<NB>& S = *reinterpret_cast<GemmSmem<NB>*>(gemm_smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t idesc = BF ? tc::idesc_bf16(128, NB) : tc::idesc_tf32(128, NB);
    constexpr uint32_t ES = BF ? 2 : 4;          // operand element bytes
    constexpr uint32_t SBO = KS * 8 * ES;        // bytes per 8-row group of a K-major tile with K = KS
    // byte offset of element (row, k) of a K-major no-swizzle tile with K = KS
    auto koff = [](int row, int k) -> uint32_t {
        return (uint32_t)((row >> 3) * SBO + (k * ES / 16) * 128 + (row & 7) * 16 + (k * ES) % 16);
    };

    const int m0 = blockIdx.x * 128;
    const int n0 = blockIdx.y * NB;
    const int64_t kbeg = TRANS_A ? (int64_t)blockIdx.z * kchunk : 0;
    const int64_t kend = TRANS_A ? (K < kbeg + kchunk ? K : kbeg + kchunk) : K;
    const int nstage = (int)((kend - kbeg + KS - 1) / KS);

    if (warp == 0) tc::tmem_alloc(&S.tmem_slot, NB);
    if (tid == 0) {
        tc::mbar_init(tc::smem_u32(&S.mbar[0]), 1);
        tc::mbar_init(tc::smem_u32(&S.mbar[1]), 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem_slot;
    uint32_t phase_bits = 0u;  // bit b: phase of mbar[b]
    bool ok = true;

    // Stage s: K rows [k0, k0 + KS).  A operand rows = output rows m, B
    // operand rows = output columns n, both K-major (KS values per row).
    // four consecutive K values of one operand row, split into hi and lo
    auto store_split = [](unsigned char* hp, unsigned char* lp, uint32_t off, const float(&v)[4]) {
        if constexpr (BF) {
            uint32_t h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) tc::split_bf16(v[e], h[e], l[e]);
            *reinterpret_cast<uint2*>(hp + off) = make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16));
            *reinterpret_cast<uint2*>(lp + off) = make_uint2(l[0] | (l[1] << 16), l[2] | (l[3] << 16));
        } else {
            uint4 hi, lo;
            tc::split_tf32(v[0], hi.x, lo.x);
            tc::split_tf32(v[1], hi.y, lo.y);
            tc::split_tf32(v[2], hi.z, lo.z);
            tc::split_tf32(v[3], hi.w, lo.w);
            *reinterpret_cast<uint4*>(hp + off) = hi;
            *reinterpret_cast<uint4*>(lp + off) = lo;
        }
    };
    auto stage = [&](int s, int buf) {
        const int64_t k0 = kbeg + (int64_t)s * KS;
        unsigned char* ah = reinterpret_cast<unsigned char*>(S.a_hi[buf]);
        unsigned char* al = reinterpret_cast<unsigned char*>(S.a_lo[buf]);
        unsigned char* bh = reinterpret_cast<unsigned char*>(S.b_hi[buf]);
        unsigned char* bl = reinterpret_cast<unsigned char*>(S.b_lo[buf]);
        // A: 128 rows x KS.  Each task = one row, 4 consecutive k.  When K
        // is contiguous in global memory (A^T), 8 neighbouring threads take
        // 8 rows of the same 16-byte K chunk (one 128-byte row of core
        // matrices: conflict-free stores) and 4 such groups cover 64
        // contiguous bytes of each row's column (full sectors).
        // All global reads of a part are issued before its shared stores:
        // interleaved, each iteration's loads would wait for the previous
        // iteration's stores (the compiler cannot rule out aliasing).
        constexpr int AT = 128 * (KS / 4) / 128;
        float va[AT][4];
#pragma unroll
        for (int it = 0; it < AT; ++it) {
            const int task = tid + 128 * it;
            int row, k4;
            if (TRANS_A) {
                const int grp = task >> 5;
                row = (grp % 16) * 8 + (task & 7);
                k4 = ((grp / 16) * 4 + ((task >> 3) & 3)) * 4;
            } else {  // consecutive threads take consecutive rows of A
                row = task % 128;
                k4 = (task / 128) * 4;
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int64_t k = k0 + k4 + e;
                const int m = m0 + row;
                float x = 0.f;
                if (k < kend && m < M) x = TRANS_A ? A[k + (int64_t)m * lda] : A[m + k * lda];
                va[it][e] = x;
            }
        }
#pragma unroll
        for (int it = 0; it < AT; ++it) {
            const int task = tid + 128 * it;
            int row, k4;
            if (TRANS_A) {
                const int grp = task >> 5;
                row = (grp % 16) * 8 + (task & 7);
                k4 = ((grp / 16) * 4 + ((task >> 3) & 3)) * 4;
            } else {
                row = task % 128;
                k4 = (task / 128) * 4;
            }
            store_split(ah, al, koff(row, k4), va[it]);
        }
        // B: NB rows (output columns) x KS; element (n, k) = Bm[k + n*ldb],
        // in rounds of at most 8 tasks per thread (loads, then stores).
        constexpr int BT = NB * (KS / 4) / 128;
        constexpr int BR = BT < 8 ? BT : 8;
#pragma unroll
        for (int r0 = 0; r0 < BT; r0 += BR) {
            float vb[BR][4];
#pragma unroll
            for (int it = 0; it < BR; ++it) {
                const int task = tid + 128 * (r0 + it);
                const int grp = task >> 5;
                const int row = (grp % (NB / 8)) * 8 + (task & 7);
                const int k4 = ((grp / (NB / 8)) * 4 + ((task >> 3) & 3)) * 4;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int64_t k = k0 + k4 + e;
                    const int nn = n0 + row;
                    vb[it][e] = (k < kend && nn < N) ? Bm[k + (int64_t)nn * ldb] : 0.f;
                }
            }
#pragma unroll
            for (int it = 0; it < BR; ++it) {
                const int task = tid + 128 * (r0 + it);
                const int grp = task >> 5;
                const int row = (grp % (NB / 8)) * 8 + (task & 7);
                const int k4 = ((grp / (NB / 8)) * 4 + ((task >> 3) & 3)) * 4;
                store_split(bh, bl, koff(row, k4), vb[it]);
            }
        }
        tc::fence_smem_to_async();
    };
    auto issue = [&](int s, int buf) {
        const uint32_t ah = tc::smem_u32(S.a_hi[buf]), al = tc::smem_u32(S.a_lo[buf]);
        const uint32_t bh = tc::smem_u32(S.b_hi[buf]), bl = tc::smem_u32(S.b_lo[buf]);
        // one MMA covers 32 bytes of K: 8 TF32 or 16 BF16 values
#pragma unroll
        for (int ks = 0; ks < KS * (int)ES / 32; ++ks) {
            const uint32_t ko = ks * 256;
            const uint64_t dah = tc::smem_desc(ah + ko, 128, SBO), dal = tc::smem_desc(al + ko, 128, SBO);
            const uint64_t dbh = tc::smem_desc(bh + ko, 128, SBO), dbl = tc::smem_desc(bl + ko, 128, SBO);
            if constexpr (BF) {
                tc::mma_bf16(tmem, dah, dbh, idesc, (s > 0) || (ks > 0));
                tc::mma_bf16(tmem, dah, dbl, idesc, true);
                tc::mma_bf16(tmem, dal, dbh, idesc, true);
            } else {
                tc::mma_tf32(tmem, dah, dbh, idesc, (s > 0) || (ks > 0));
                tc::mma_tf32(tmem, dah, dbl, idesc, true);
                tc::mma_tf32(tmem, dal, dbh, idesc, true);
            }
        }
        tc::mma_commit(tc::smem_u32(&S.mbar[buf]));
    };

    // pend: buffers whose committed MMA group this thread has not yet seen
    // complete (at most one group per buffer is outstanding at a time);
    // phase_bits: the parity of each buffer's next phase.  A wait that
    // succeeds consumes its phase; one that gives up leaves it pending.
    uint32_t pend = 0;
#define TSQR_WAIT_BUF(w, b, n)                                                                  \
    do {                                                                                        \
        const int b_ = (b);                                                                     \
        w = tc::mbar_wait(tc::smem_u32(&S.mbar[b_]), (phase_bits >> b_) & 1u, (n));             \
        if (w) {                                                                                \
            phase_bits ^= 1u << b_;                                                             \
            pend &= ~(1u << b_);                                                                \
        }                                                                                       \
    } while (0)
    if (nstage > 0) stage(0, 0);
    for (int s = 0; s < nstage && ok; ++s) {
        const int buf = s & 1;
        tc::fence_before_sync();
        __syncthreads();  // stage s is in shared memory
        if (tid == 0) {
            tc::fence_after_sync();
            issue(s, buf);
        }
        pend |= 1u << buf;
        if (s + 1 < nstage) {
            // buffer buf^1 was read by the MMAs of stage s-1: wait for them
            bool waited = true;
            if (s >= 1) TSQR_WAIT_BUF(waited, buf ^ 1, tries);
            if (__syncthreads_or(!waited)) {
                ok = false;
                break;
            }
            stage(s + 1, buf ^ 1);
        }
    }
    // wait for the last two stages' MMAs (in order of commit)
    if (ok && nstage > 0) {
        bool w0 = true, w1;
        if (nstage >= 2) TSQR_WAIT_BUF(w0, (nstage - 2) & 1, tries);
        TSQR_WAIT_BUF(w1, (nstage - 1) & 1, tries);
        if (__syncthreads_or(!(w0 && w1))) ok = false;
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // MMAs still in flight write TMEM: give them a full bounded wait to
        // retire before it is freed
        bool w;
        if (pend & 1u) TSQR_WAIT_BUF(w, 0, tc::kMbarTries);
        if (pend & 2u) TSQR_WAIT_BUF(w, 1, tc::kMbarTries);
        (void)w;
    } else {
        tc::fence_after_sync();
        const int m = m0 + 32 * warp + (tid & 31);
        float* Cz = TRANS_A ? C + (int64_t)blockIdx.z * M * N : C;
        const int64_t ldz = TRANS_A ? M : ldc;
#pragma unroll 2
        for (int c8 = 0; c8 < NB; c8 += 8) {
            float d[8];
            tc::tmem_ld8(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c8, d);
            tc::tmem_ld_wait();
            if (m < M) {
                if (TRANS_A) {
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int nn = n0 + c8 + e;
                        if (nn < N) Cz[m + (int64_t)nn * ldz] = nstage > 0 ? d[e] : 0.f;
                    }
                } else if (nstage > 0) {
                    // all eight loads first, so their latencies overlap
                    float c[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int nn = n0 + c8 + e;
                        c[e] = (nn < N) ? Cz[m + (int64_t)nn * ldz] : 0.f;
                    }
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        const int nn = n0 + c8 + e;
                        if (nn < N) Cz[m + (int64_t)nn * ldz] = c[e] + alpha * d[e];
                    }
                }
            }
        }
    }
#undef TSQR_WAIT_BUF
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, NB);
}

template <bool TRANS_A, int NB, bool BF>
void launch_gemm(dim3 grid, int M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
                 float* C, int64_t ldc, float alpha, int64_t kchunk, int* err, cudaStream_t s) {
    constexpr size_t smem = sizeof(GemmSmem<NB>) + 1024;
    static PerDeviceOnce attr;
    attr.run([] {
        cudaFuncSetAttribute(tc_gemm_kernel<TRANS_A, NB, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    });
    launch_pdl(tc_gemm_kernel<TRANS_A, NB, BF>, grid, dim3(128), smem, s, M, N, K, A, lda, B, ldb, C, ldc, alpha,
               kchunk, err, wait_tries().load(std::memory_order_relaxed));
}

template <bool TRANS_A, bool BF>
void launch_nb(int nb, dim3 g, int M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
               float* C, int64_t ldc, float alpha, int64_t kchunk, int* err, cudaStream_t s) {
    switch (nb) {
        case 32: launch_gemm<TRANS_A, 32, BF>(g, M, N, K, A, lda, B, ldb, C, ldc, alpha, kchunk, err, s); break;
        case 64: launch_gemm<TRANS_A, 64, BF>(g, M, N, K, A, lda, B, ldb, C, ldc, alpha, kchunk, err, s); break;
        case 128: launch_gemm<TRANS_A, 128, BF>(g, M, N, K, A, lda, B, ldb, C, ldc, alpha, kchunk, err, s); break;
        default: launch_gemm<TRANS_A, 256, BF>(g, M, N, K, A, lda, B, ldb, C, ldc, alpha, kchunk, err, s); break;
    }
}

int nb_for(int N) { return N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256)); }

// ---------------------------------------------------------------------------
// P_z = A^T B (TF32x3) with the operands fed by TMA.  A (K x M) and B (K x N)
// are column-major, so each is K-major as an MMA operand: a 32-row stage of
// K arrives as boxes of 32 x 128 (A) and 32 x NB (B) with the 128-byte
// swizzle, which is the layout the MMA reads (smem_desc_sw128).  The raw
// FP32 tile is the hi operand (TF32 reads the top 19 bits); one pass of the
// CTA (256 threads) writes lo = x - trunc(x) beside it at the same offsets,
// and one thread issues hi*hi + hi*lo + lo*hi for the 4 K steps of 8.  Two
// stages: the copy of stage s+2 is issued once the MMAs of stage s have
// read its buffers.  The epilogue splits the TMEM read-back by column
// halves: warp w reads lanes 32 (w % 4) .. +31 of half w / 4.  Every wait
// is bounded; a CTA whose wait gives up sets the status word, waits (with
// the full limit) for its copies and MMAs in flight, frees its TMEM and
// stops.
template <int NB>
struct TnTma {
    static constexpr int A_BYTES = 128 * 128;             // 128 rows of 32 FP32
    static constexpr int B_BYTES = NB * 128;
    static constexpr int RAW = A_BYTES + B_BYTES;          // raw A | raw B
    static constexpr int STAGE = 2 * RAW;                  // then lo A | lo B
    static constexpr size_t SMEM = 2 * (size_t)STAGE + 1024;
};

template <int NB>
__global__ void __launch_bounds__(256, 1)
    tc_tn_tma_kernel(int M, int N, int64_t K, int64_t kchunk, float* __restrict__ P,
                     const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int* err,
                     int tries) {
    pdl_begin();
    using L = TnTma<NB>;
    extern __shared__ unsigned char tn_smem[];
    __shared__ unsigned long long full[2], mmad[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int t0_failed;
    unsigned char* base = tn_smem + ((1024 - (tc::smem_u32(tn_smem) & 1023)) & 1023);
    const uint32_t sbase = tc::smem_u32(base);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * NB;
    const int64_t kbeg = (int64_t)blockIdx.z * kchunk;
    const int64_t kend = K < kbeg + kchunk ? K : kbeg + kchunk;
    const int nst = kend > kbeg ? (int)((kend - kbeg + 31) / 32) : 0;
    constexpr uint32_t idesc = tc::idesc_tf32(128, NB);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, NB);
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(tc::smem_u32(&full[b]), 1);
            tc::mbar_init(tc::smem_u32(&mmad[b]), 1);
        }
        tc::fence_mbar_init();
        t0_failed = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    // thread 0's record of what is in flight: copies issued (stages
    // [0, issued)), MMA groups committed ([0, committed)) and waited ([0, mwaited))
    int issued = 0, committed = 0, mwaited = 0;
    auto issue = [&](int s) {
        const int b = s & 1;
        const uint32_t dst = sbase + b * L::STAGE, mb = tc::smem_u32(&full[b]);
        const int x = (int)(kbeg + 32 * (int64_t)s);
        tc::fence_smem_to_async();
        tc::mbar_arrive_expect_tx(mb, L::RAW);
        tc::tma_load_2d(dst, &ta, x, m0, mb);
        tc::tma_load_2d(dst + L::A_BYTES, &tb, x, n0, mb);
        issued = s + 1;
    };
    if (tid == 0) {
        if (nst > 0) issue(0);
        if (nst > 1) issue(1);
    }
    bool ok = true;
    int s = 0;
    for (; s < nst; ++s) {
        const int b = s & 1;
        const bool w = tc::mbar_wait(tc::smem_u32(&full[b]), (uint32_t)(s >> 1) & 1u, tries);
        if (__syncthreads_or(!w || t0_failed)) {
            ok = false;
            break;
        }
        // lo = x - trunc_tf32(x), written beside the raw tile
        {
            const uint4* src = reinterpret_cast<const uint4*>(base + b * L::STAGE);
            uint4* dst = reinterpret_cast<uint4*>(base + b * L::STAGE + L::RAW);
#pragma unroll 4
            for (int i = tid; i < L::RAW / 16; i += 256) {
                const uint4 x = src[i];
                uint4 lo;
                lo.x = __float_as_uint(__uint_as_float(x.x) - __uint_as_float(x.x & 0xFFFFE000u));
                lo.y = __float_as_uint(__uint_as_float(x.y) - __uint_as_float(x.y & 0xFFFFE000u));
                lo.z = __float_as_uint(__uint_as_float(x.z) - __uint_as_float(x.z & 0xFFFFE000u));
                lo.w = __float_as_uint(__uint_as_float(x.w) - __uint_as_float(x.w & 0xFFFFE000u));
                dst[i] = lo;
            }
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            const uint32_t st = sbase + b * L::STAGE;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint32_t ko = ks * 32;
                const uint64_t ah = tc::smem_desc_sw128(st + ko), bh = tc::smem_desc_sw128(st + L::A_BYTES + ko);
                const uint64_t al = tc::smem_desc_sw128(st + L::RAW + ko),
                               bl = tc::smem_desc_sw128(st + L::RAW + L::A_BYTES + ko);
                tc::mma_tf32(tmem, ah, bh, idesc, (s > 0) || (ks > 0));
                tc::mma_tf32(tmem, ah, bl, idesc, true);
                tc::mma_tf32(tmem, al, bh, idesc, true);
            }
            tc::mma_commit(tc::smem_u32(&mmad[b]));
            committed = s + 1;
            if (s + 2 < nst) {
                // the copy of stage s+2 overwrites buffer b: the MMAs of
                // stage s read it
                if (tc::mbar_wait(tc::smem_u32(&mmad[b]), (uint32_t)(s >> 1) & 1u, tries)) {
                    mwaited = s + 1;
                    issue(s + 2);
                } else {
                    t0_failed = 1;
                }
            }
        }
    }
    if (ok && nst > 0) {
        // the last one or two MMA groups (never waited for in the loop)
        bool w0 = true;
        const int first = nst >= 2 ? nst - 2 : 0;
        for (int q = first; q < nst; ++q)
            w0 = tc::mbar_wait(tc::smem_u32(&mmad[q & 1]), (uint32_t)(q >> 1) & 1u, tries) && w0;
        if (__syncthreads_or(!w0)) ok = false;
        else if (tid == 0) mwaited = nst;
    }
    if (!ok) {
        if (tid == 0) {
            if (err) atomicExch(err, 1);
            // every copy and MMA group still in flight, with the full limit
            for (int q = s; q < issued; ++q)
                (void)tc::mbar_wait(tc::smem_u32(&full[q & 1]), (uint32_t)(q >> 1) & 1u);
            for (int q = mwaited; q < committed; ++q)
                (void)tc::mbar_wait(tc::smem_u32(&mmad[q & 1]), (uint32_t)(q >> 1) & 1u);
        }
    } else {
        // warp w: TMEM lanes 32 (w % 4) .. +31, columns of half w / 4
        tc::fence_after_sync();
        const int m = m0 + 32 * (warp & 3) + (tid & 31);
        float* Pz = P + (int64_t)blockIdx.z * M * N;
        constexpr int HALF = NB / 2;
        const int cb = (warp >> 2) * HALF;
#pragma unroll 2
        for (int c8 = 0; c8 < HALF; c8 += 8) {
            float d[8];
            tc::tmem_ld8(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(cb + c8), d);
            tc::tmem_ld_wait();
            if (m < M) {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int nn = n0 + cb + c8 + e;
                    if (nn < N) Pz[m + (int64_t)nn * M] = nst > 0 ? d[e] : 0.f;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, NB);
}

// ---------------------------------------------------------------------------
// C (M x N) += alpha A (M x K) B (K x N), TF32x3, A tall (the blocked QR's
// update A2 -= A1 X).  B is K-major in memory (X column-major) and arrives by
// TMA in the MMA's 128-byte swizzled K-major layout, raw FP32 as hi, lo
// written beside it.  A is MN-major in memory (rows contiguous): each
// 128 x 32 stage arrives as four 32 x 32 boxes with the 128-byte swizzle
// (element (r, k) at (r/32) 4096 + k 128 + 16 ((r%32)/4 ^ k%8) + 4 (r%4)),
// and the CTA rewrites it as K-major hi and lo tiles (element (r, k) at
// r 128 + 16 (k/4 ^ r%8) + 4 (k%4)): lane l takes K index l and 4 rows per
// 16-byte read, so the reads take the four wavefronts a 512-byte warp read
// needs anyway and each 4-byte store of the warp hits 32 distinct banks.
// hi = x rounded to TF32, lo = the rest, for B as well, so that a
// copy's buffer is free once the CTA has rewritten it: the copies run in a
// ring of three stages (the copy of step t+3 is issued right after step t's
// rewrite), the operand tiles in two buffers (step t's rewrite waits for the
// MMAs of step t-2).  A persistent CTA (one per SM, 256 threads: warp w
// rewrites row groups 4w..4w+3) walks 128-row blocks; a block's K stages
// accumulate in TMEM, and its epilogue (warp w: TMEM lanes 32 (w % 4) ..
// +31, columns of half w / 4) reads C 16 columns at a time, adds alpha D
// and writes it back.  Bounded waits as in the projection kernel.
template <int NB>
struct NnTma {
    static constexpr int A_RAW = 128 * 128;            // four 32 x 32 boxes
    static constexpr int B_RAW = NB * 128;
    static constexpr int RAW = A_RAW + B_RAW;          // one raw stage (TMA destination)
    static constexpr int A_OP = 128 * 128;             // one K-major operand tile of A
    static constexpr int B_OP = NB * 128;
    static constexpr int OPS = 2 * A_OP + 2 * B_OP;    // A hi | A lo | B hi | B lo
    static constexpr int NRAW = 3;                     // raw ring depth
    static constexpr size_t SMEM = NRAW * (size_t)RAW + 2 * (size_t)OPS + 1024;
};

template <int NB>
__global__ void __launch_bounds__(256, 1)
    tc_nn_tma_kernel(int64_t M, int N, int K, float alpha, float* __restrict__ C, int64_t ldc,
                     const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int* err,
                     int tries) {
    pdl_begin();
    using L = NnTma<NB>;
    extern __shared__ unsigned char nn_smem[];
    __shared__ unsigned long long full[L::NRAW], mmad[2];
    __shared__ uint32_t tmem_slot;
    unsigned char* base = nn_smem + ((1024 - (tc::smem_u32(nn_smem) & 1023)) & 1023);
    const uint32_t sbase = tc::smem_u32(base);
    unsigned char* opsbase = base + L::NRAW * L::RAW;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.x * NB;
    const int64_t nblk = (M + 127) / 128;
    const int nks = (K + 31) / 32;
    // this CTA's blocks: blockIdx.y, + gridDim.y, ...; steps t = (block j, stage s)
    const int64_t myblk = nblk > blockIdx.y ? (nblk - 1 - blockIdx.y) / gridDim.y + 1 : 0;
    const int64_t T = myblk * nks;
    constexpr uint32_t idesc = tc::idesc_tf32(128, NB);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, NB);
    if (tid == 0) {
        for (int b = 0; b < L::NRAW; ++b) tc::mbar_init(tc::smem_u32(&full[b]), 1);
        for (int b = 0; b < 2; ++b) tc::mbar_init(tc::smem_u32(&mmad[b]), 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    int64_t issued = 0, committed = 0;  // thread 0: copies issued for steps [0, issued), MMA groups committed
    auto issue = [&](int64_t t) {
        const int rb = (int)(t % L::NRAW);
        const int64_t j = t / nks;
        const int s = (int)(t % nks);
        const int r0 = (int)((blockIdx.y + j * gridDim.y) * 128);
        const uint32_t dst = sbase + rb * L::RAW, mb = tc::smem_u32(&full[rb]);
        tc::fence_smem_to_async();
        tc::mbar_arrive_expect_tx(mb, L::RAW);
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::tma_load_2d(dst + q * 4096, &ta, r0 + 32 * q, 32 * s, mb);
        tc::tma_load_2d(dst + L::A_RAW, &tb, 32 * s, n0, mb);
        issued = t + 1;
    };
    if (tid == 0)
        for (int64_t q = 0; q < L::NRAW && q < T; ++q) issue(q);
    bool ok = true;
    int64_t t = 0;
    for (; t < T; ++t) {
        const int rb = (int)(t % L::NRAW), ob = (int)(t & 1);
        const int s = (int)(t % nks);
        // the stage's copy has landed, and the MMAs of step t-2 (which read
        // operand buffer ob) are done
        bool w = tc::mbar_wait(tc::smem_u32(&full[rb]), (uint32_t)((t / L::NRAW) & 1), tries);
        if (t >= 2) w = tc::mbar_wait(tc::smem_u32(&mmad[ob]), (uint32_t)((t - 2) >> 1) & 1u, tries) && w;
        if (__syncthreads_or(!w)) {
            ok = false;
            break;
        }
        const unsigned char* ra = base + rb * L::RAW;
        unsigned char* ah = opsbase + ob * L::OPS;
        unsigned char* al = ah + L::A_OP;
        unsigned char* bh = al + L::A_OP;
        unsigned char* bl = bh + L::B_OP;
        {
            // A: MN-major raw -> K-major hi, lo; lane = K index, 4 groups of 4 rows per warp
            const int k = lane;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int g = warp * 4 + i, r = 4 * g;  // rows r .. r + 3
                const uint4 x = *reinterpret_cast<const uint4*>(ra + (r >> 5) * 4096 + k * 128 +
                                                                ((((r & 31) >> 2) ^ (k & 7)) << 4));
                const uint32_t xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int rr = r + q;
                    const uint32_t off = rr * 128 + ((((k >> 2) ^ (rr & 7))) << 4) + (k & 3) * 4;
                    uint32_t hi, lo;
                    tc::split_tf32(__uint_as_float(xv[q]), hi, lo);
                    *reinterpret_cast<uint32_t*>(ah + off) = hi;
                    *reinterpret_cast<uint32_t*>(al + off) = lo;
                }
            }
            // B: already K-major; hi and lo at the same offsets
            const uint4* rbp = reinterpret_cast<const uint4*>(ra + L::A_RAW);
            uint4* bhp = reinterpret_cast<uint4*>(bh);
            uint4* blp = reinterpret_cast<uint4*>(bl);
#pragma unroll 4
            for (int i = tid; i < L::B_RAW / 16; i += 256) {
                const uint4 x = rbp[i];
                uint4 h, lo;
                tc::split_tf32(__uint_as_float(x.x), h.x, lo.x);
                tc::split_tf32(__uint_as_float(x.y), h.y, lo.y);
                tc::split_tf32(__uint_as_float(x.z), h.z, lo.z);
                tc::split_tf32(__uint_as_float(x.w), h.w, lo.w);
                bhp[i] = h;
                blp[i] = lo;
            }
        }
        tc::fence_smem_to_async();
        tc::fence_before_sync();
        __syncthreads();  // raw buffer rb consumed, operand buffer ob written
        if (tid == 0) {
            tc::fence_after_sync();
            if (t + L::NRAW < T) issue(t + L::NRAW);
            const uint32_t so = tc::smem_u32(ah);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                const uint32_t ko = ks * 32;
                const uint64_t dah = tc::smem_desc_sw128(so + ko);
                const uint64_t dal = tc::smem_desc_sw128(so + L::A_OP + ko);
                const uint64_t dbh = tc::smem_desc_sw128(so + 2 * L::A_OP + ko);
                const uint64_t dbl = tc::smem_desc_sw128(so + 2 * L::A_OP + L::B_OP + ko);
                tc::mma_tf32(tmem, dah, dbh, idesc, (s > 0) || (ks > 0));
                tc::mma_tf32(tmem, dah, dbl, idesc, true);
                tc::mma_tf32(tmem, dal, dbh, idesc, true);
            }
            tc::mma_commit(tc::smem_u32(&mmad[ob]));
            committed = t + 1;
        }
        if (s == nks - 1) {
            // the block's last stage: its MMAs done, C += alpha D
            const bool wd = tc::mbar_wait(tc::smem_u32(&mmad[ob]), (uint32_t)(t >> 1) & 1u, tries);
            if (__syncthreads_or(!wd)) {
                ok = false;
                ++t;  // stage t was consumed
                break;
            }
            // warp w: TMEM lanes 32 (w % 4) .. +31, columns of half w / 4
            tc::fence_after_sync();
            const int64_t j = t / nks;
            const int64_t m = (blockIdx.y + j * gridDim.y) * 128 + 32 * (warp & 3) + lane;
            constexpr int HALF = NB / 2;
            const int cb = (warp >> 2) * HALF;
#pragma unroll 1
            for (int c16 = 0; c16 < HALF; c16 += 16) {
                // 16 columns per round: the TMEM reads and the 16 loads of C
                // are all in flight before the first store
                float d[16], c[16];
#pragma unroll
                for (int c8 = 0; c8 < 16; c8 += 8)
                    tc::tmem_ld8(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(cb + c16 + c8),
                                 *reinterpret_cast<float(*)[8]>(d + c8));
                if (m < M) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        const int nn = n0 + cb + c16 + e;
                        c[e] = (nn < N) ? C[m + (int64_t)nn * ldc] : 0.f;
                    }
                }
                tc::tmem_ld_wait();
                if (m < M) {
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        const int nn = n0 + cb + c16 + e;
                        if (nn < N) C[m + (int64_t)nn * ldc] = c[e] + alpha * d[e];
                    }
                }
            }
            tc::fence_before_sync();
            __syncthreads();  // TMEM is read: the next block's MMAs may overwrite it
        }
    }
    if (!ok) {
        if (tid == 0) {
            if (err) atomicExch(err, 1);
            // every copy and MMA group still in flight, with the full limit
            for (int64_t q = t; q < issued; ++q)
                (void)tc::mbar_wait(tc::smem_u32(&full[q % L::NRAW]), (uint32_t)((q / L::NRAW) & 1));
            for (int64_t q = committed >= 2 ? committed - 2 : 0; q < committed; ++q)
                (void)tc::mbar_wait(tc::smem_u32(&mmad[q & 1]), (uint32_t)(q >> 1) & 1u);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, NB);
}

template <int NB>
bool launch_nn_tma(int64_t M, int N, int K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                   float* C, int64_t ldc, int* err, cudaStream_t s) {
    CUtensorMap ta, tb;
    if (M + 128 > INT32_MAX || !tensor_map_f32(&ta, A, lda, M, K, 32, 32, true) ||
        !tensor_map_f32(&tb, B, ldb, K, N, 32, NB, true))
        return false;
    static PerDeviceOnce attr;
    attr.run([] {
        cudaFuncSetAttribute(tc_nn_tma_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)NnTma<NB>::SMEM);
    });
    const int ntn = (N + NB - 1) / NB;
    const int64_t nblk = (M + 127) / 128;
    const int gy = (int)std::max<int64_t>(1, std::min<int64_t>(nblk, (device_sm_count() + ntn - 1) / ntn));
    launch_pdl(tc_nn_tma_kernel<NB>, dim3((unsigned)ntn, (unsigned)gy), dim3(256), NnTma<NB>::SMEM, s, M, N, K,
               alpha, C, ldc, ta, tb, err, wait_tries().load(std::memory_order_relaxed));
    return true;
}

template <int NB>
bool launch_tn_tma(dim3 g, int M, int N, int64_t K, int64_t kchunk, const float* A, int64_t lda, const float* B,
                   int64_t ldb, float* P, int* err, cudaStream_t s) {
    CUtensorMap ta, tb;
    if (K + 64 > INT32_MAX || !tensor_map_f32(&ta, A, lda, K, M, 32, 128, true) ||
        !tensor_map_f32(&tb, B, ldb, K, N, 32, NB, true))
        return false;
    static PerDeviceOnce attr;
    attr.run([] {
        cudaFuncSetAttribute(tc_tn_tma_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)TnTma<NB>::SMEM);
    });
    launch_pdl(tc_tn_tma_kernel<NB>, g, dim3(256), TnTma<NB>::SMEM, s, M, N, K, kchunk, P, ta, tb, err,
               wait_tries().load(std::memory_order_relaxed));
    return true;
}

}  // namespace

int tc_tn_splits(int64_t M, int64_t N, int64_t K) {
    // one wave of one CTA per SM on GB300's 152 SMs (the TMA form's 193 KB
    // of shared memory); the workspace query uses the same count
    const int64_t tiles = ((M + 127) / 128) * ((N + 255) / 256);
    int64_t nz = std::max<int64_t>(1, (152 + tiles - 1) / tiles);
    nz = std::min<int64_t>(nz, std::max<int64_t>(1, K / 1024));
    return (int)nz;
}

// P_z = A^T B over K-chunks (M, N <= 256 per launch dimension); P holds
// nz * M * N floats.  Returns the number of partial sums written.  bf16:
// BF16x3 products instead of TF32x3.
int tc_gemm_tn(int M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb, float* P, int* err,
               cudaStream_t s, bool bf16) {
    const int nz = tc_tn_splits(M, N, K);
    int64_t kchunk = (K + nz - 1) / nz;
    kchunk = (kchunk + KS - 1) / KS * KS;
    const int nzr = (int)((K + kchunk - 1) / kchunk);
    const int nb = nb_for(std::min(N, 256));
    dim3 g((unsigned)((M + 127) / 128), (unsigned)((N + nb - 1) / nb), (unsigned)nzr);
    if (bf16) {
        launch_nb<true, true>(nb, g, M, N, K, A, lda, B, ldb, P, M, 1.f, kchunk, err, s);
        return nzr;
    }
    bool done = false;
    switch (nb) {
        case 32: done = launch_tn_tma<32>(g, M, N, K, kchunk, A, lda, B, ldb, P, err, s); break;
        case 64: done = launch_tn_tma<64>(g, M, N, K, kchunk, A, lda, B, ldb, P, err, s); break;
        case 128: done = launch_tn_tma<128>(g, M, N, K, kchunk, A, lda, B, ldb, P, err, s); break;
        default: done = launch_tn_tma<256>(g, M, N, K, kchunk, A, lda, B, ldb, P, err, s); break;
    }
    if (!done) launch_nb<true, false>(nb, g, M, N, K, A, lda, B, ldb, P, M, 1.f, kchunk, err, s);
    return nzr;
}

// C (M x N) += alpha * A (M x K) * B (K x N), K and N small (<= 256 per N
// block).  bf16: BF16x3 products instead of TF32x3.
void tc_gemm_nn(int64_t M, int N, int K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                float* C, int64_t ldc, int* err, cudaStream_t s, bool bf16) {
    const int nb = nb_for(std::min(N, 256));
    dim3 g((unsigned)((M + 127) / 128), (unsigned)((N + nb - 1) / nb), 1);
    if (bf16) {
        launch_nb<false, true>(nb, g, (int)M, N, K, A, lda, B, ldb, C, ldc, alpha, 0, err, s);
        return;
    }
    // the TMA-fed form in N tiles of at most 128 (225 KB of shared memory)
    bool done = false;
    switch (nb) {
        case 32: done = launch_nn_tma<32>(M, N, K, alpha, A, lda, B, ldb, C, ldc, err, s); break;
        case 64: done = launch_nn_tma<64>(M, N, K, alpha, A, lda, B, ldb, C, ldc, err, s); break;
        default: done = launch_nn_tma<128>(M, N, K, alpha, A, lda, B, ldb, C, ldc, err, s); break;
    }
    if (!done) launch_nb<false, false>(nb, g, (int)M, N, K, A, lda, B, ldb, C, ldc, alpha, 0, err, s);
}

}  // namespace tsqr
