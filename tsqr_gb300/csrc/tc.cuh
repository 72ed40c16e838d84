// tc.cuh -- Blackwell (sm_103a) tensor-core primitives in inline PTX:
// tcgen05 MMA with TMEM accumulators, shared-memory matrix descriptors,
// mbarriers with bounded waits, and the TF32 hi/lo split.
//
// Operand layout used throughout: K-major, no swizzle.  A core matrix is 8
// rows (M or N) x 16 bytes of K (4 TF32 values) stored as 128 contiguous
// bytes (row r at +16 r).  Core matrices adjacent in K are LBO = 128 bytes
// apart; row groups of 8 are SBO bytes apart (SBO = K/4 * 128 for a tile
// stored K-contiguous).  Element (row, k) of such a tile therefore sits at
// byte  (row/8)*SBO + (k/4)*128 + (row%8)*16 + (k%4)*4.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tsqr {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row, k) in a K-major, no-swizzle operand tile with
// K columns (K % 4 == 0).
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int K) {
    return (uint32_t)((row >> 3) * (K * 32) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor (tcgen05 format): start address, leading
// byte offset (K direction), stride byte offset (8-row groups), version 1,
// no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, lbo mode 0, layout 0 = no swizzle
}

// The same for a K-major operand in the 128-byte swizzled layout that TMA
// writes with CU_TENSOR_MAP_SWIZZLE_128B: rows of 128 bytes of K, 8-row
// groups 1024 bytes apart (SBO), the leading offset unused (encoded 1),
// layout type 2 (128-byte swizzle) in bits 61-63.  The buffer must be
// 1024-byte aligned; a K step inside the 128-byte row advances the start
// address, and the hardware applies the swizzle to the computed addresses.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;            // leading byte offset: unused for this layout
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;            // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M x N tile.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4)                       // D format F32
           | (2u << 7)                     // A format TF32
           | (2u << 10)                    // B format TF32
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// Instruction descriptor, kind::f16 with BF16 A and B (both the same type),
// FP32 accumulator, both K-major, M x N tile.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)                       // D format F32
           | (1u << 7)                     // A format BF16
           | (1u << 10)                    // B format BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// D[tmem] (+)= A[smem] * B[smem], BF16 operands (K = 16), issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// D[tmem] (+)= A[smem] * B[smem], issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// Arrive on an mbarrier once all previously issued MMAs of this thread finish.
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}

// TMEM allocation by one full warp; the TMEM address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Make generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 32 lanes x 32 bits, 8 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// mbarriers
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// Bounded wait for phase `parity` of an mbarrier.  Each try_wait may suspend
// the thread for a hardware-defined time; after `tries` unsuccessful tries
// (kMbarTries: seconds) it gives up and returns false instead of spinning
// forever.  tries = 0 gives up at once.
constexpr int kMbarTries = 1 << 24;
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int tries = kMbarTries) {
    for (int it = 0; it < tries; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// TMA: announce `bytes` of transactions on an mbarrier (and arrive once).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
}
// TMA: 2D tiled load of the box at coordinates (x, y) of the tensor map into
// shared memory, completing as transactions on `mbar`.  x (the innermost,
// contiguous coordinate) times the element size must be a multiple of 16.
__device__ __forceinline__ void tma_load_2d(uint32_t smem_dst, const void* tmap, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(smem_dst),
        "l"(tmap), "r"(x), "r"(y), "r"(mbar)
        : "memory");
}

// TF32 split: hi = x rounded to TF32 (round to nearest, ties away), lo = the
// rounded remainder.  hi*hi + hi*lo + lo*hi reproduces an FP32 product to
// about 2^-21 relative.
__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
}

// BF16 split: hi = x rounded to BF16 (nearest even), lo = the remainder
// rounded to BF16; hi*hi + hi*lo + lo*hi keeps about 2^-16 relative of an
// FP32 product (the BF16x3 form).  Returned as the 16-bit patterns.
__device__ __forceinline__ uint32_t to_bf16(float x) {
    unsigned short h;
    asm("cvt.rn.bf16.f32 %0, %1;\n" : "=h"(h) : "f"(x));
    return (uint32_t)h;
}
__device__ __forceinline__ void split_bf16(float x, uint32_t& hi, uint32_t& lo) {
    hi = to_bf16(x);
    lo = to_bf16(x - __uint_as_float(hi << 16));
}

}  // namespace tc
}  // namespace tsqr
