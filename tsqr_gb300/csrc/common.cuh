// common.cuh -- small device helpers shared by the TSQR kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tsqr {

constexpr unsigned kFull = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) v += __shfl_xor_sync(kFull, v, s);
    return v;
}

// Warp transpose-reduction of NV per-lane partial sums (NV in 8..64, a power
// of two).  Round s halves the live values: lanes with bit s set keep the
// upper half and receive the partner's upper half, the others keep the lower
// half; once one value is left, the remaining rounds are plain butterflies.
// Costs NV-1 shuffles per lane for NV <= 32 (vs 5*NV for NV butterflies).
// On return the warp sums sit in p[0 .. max(NV/32,1)) of each lane:
//   NV >= 32: lane l holds indices l*(NV/32) + k, k < NV/32;
//   NV <  32: lane l holds index l / (32/NV) (all 32/NV lanes of a group).
template <int CNT, int S>
struct TransposeRound {
    template <typename T, int NV>
    static __device__ __forceinline__ void run(T (&p)[NV], int lane) {
        if constexpr (CNT > 1) {
            constexpr int H = CNT / 2;
            const bool up = (lane & S) != 0;
#pragma unroll
            for (int k = 0; k < H; ++k) {
                T send = up ? p[k] : p[k + H];
                T keep = up ? p[k + H] : p[k];
                p[k] = keep + __shfl_xor_sync(kFull, send, S);
            }
            if constexpr (S > 1) TransposeRound<H, S / 2>::run(p, lane);
        } else {
            p[0] += __shfl_xor_sync(kFull, p[0], S);
            if constexpr (S > 1) TransposeRound<1, S / 2>::run(p, lane);
        }
    }
};

// Reduce NV partials across the warp and store the warp's NV sums to row[].
template <typename T, int NV>
__device__ __forceinline__ void warp_reduce_to_smem(T (&p)[NV], T* row, int lane) {
    TransposeRound<NV, 16>::run(p, lane);
    if constexpr (NV >= 32) {
        constexpr int K = NV / 32;
#pragma unroll
        for (int k = 0; k < K; ++k) row[lane * K + k] = p[k];
    } else {
        constexpr int G = 32 / NV;
        if ((lane % G) == 0) row[lane / G] = p[0];
    }
}

// Same result as warp_reduce_to_smem, through a per-warp shared-memory
// transpose instead of shuffles: every lane stores its NV partials as one
// padded row (16-byte stores), then lane l sums column l (and l + 32 for
// NV = 64).  The row stride NV + 4 keeps both the row stores and the column
// loads free of bank conflicts.  About 8 + 32 + 31 instructions per lane for
// NV = 32 instead of 31 shuffles, 31 adds and 62 selects.  FP32 only.
template <int NV>
__host__ __device__ constexpr int xpose_stride() {
    return NV + 4;
}
template <int NV>
__device__ __forceinline__ void warp_reduce_to_smem_x(float (&p)[NV], float* row, float* scratch, int lane) {
    constexpr int SP = xpose_stride<NV>();
    float* mine = scratch + lane * SP;
#pragma unroll
    for (int c = 0; c < NV; c += 4) *reinterpret_cast<float4*>(mine + c) = make_float4(p[c], p[c + 1], p[c + 2], p[c + 3]);
    __syncwarp();
#pragma unroll
    for (int half = 0; half < (NV + 31) / 32; ++half) {
        const int idx = lane + 32 * half;
        if (idx < NV) {
            // pairwise (tree) sum: depth 5 instead of a 31-add chain
            float a[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) a[r] = scratch[r * SP + idx];
#pragma unroll
            for (int w = 16; w >= 1; w >>= 1)
#pragma unroll
                for (int r = 0; r < w; ++r) a[r] += a[r + w];
            row[idx] = a[0];
        }
    }
    __syncwarp();
}

// 1/x rounded to nearest (FP32: one reciprocal instruction sequence instead
// of the general division routine).
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

// Programmatic dependent launch.  A kernel of a call's chain is launched
// with launch_pdl (internal.h), so it may be scheduled while the previous
// kernel of its stream is still running.  It calls pdl_begin() first: that
// lets the kernel after it be scheduled too (once every CTA of this grid has
// got this far), then waits until the previous grid has completed and its
// memory is visible.  Nothing before it touches global memory.  Launched
// without the attribute, both instructions do nothing.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

}  // namespace tsqr
