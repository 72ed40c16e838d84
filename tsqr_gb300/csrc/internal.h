// internal.h -- declarations shared by the library's translation units.
#pragma once
#include <cuda.h>  // CUtensorMap (the type only; the encoder is looked up at run time)
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/tsqr_gb300.h"

namespace tsqr {

// Function attributes (the dynamic shared-memory limit) and device
// properties belong to one device's context, so the caches below keep one
// entry per device: a process that drives several GPUs sets each one up.
constexpr int kMaxDevices = 64;

inline int current_device() {
    int dev = 0;
    return cudaGetDevice(&dev) == cudaSuccess ? dev : 0;
}

// Runs f() once per device (the current device at the call); thread-safe.
// Devices past kMaxDevices are not cached: f() runs on every call.
class PerDeviceOnce {
  public:
    template <typename F>
    void run(F&& f) {
        const int dev = current_device();
        if (dev < 0 || dev >= kMaxDevices) {
            f();
            return;
        }
        const uint64_t bit = 1ull << dev;
        if (done_.load(std::memory_order_acquire) & bit) return;
        std::lock_guard<std::mutex> lk(mu_);
        if (done_.load(std::memory_order_relaxed) & bit) return;
        f();
        done_.fetch_or(bit, std::memory_order_release);
    }

  private:
    std::atomic<uint64_t> done_{0};
    std::mutex mu_;
};

// Launches kernel<<<grid, block, smem, s>>>(args...) with programmatic
// stream serialization: the kernel may be scheduled before the previous
// kernel of the stream has finished, and waits for it in pdl_begin()
// (common.cuh), which every kernel launched this way calls first.  This
// hides the launch and prologue of each kernel of a call's chain behind the
// tail of the one before.
// A call whose kernels wait on copies of another stream (the host-buffer
// entry points) turns the attribute off for its launches with a PdlOff
// scope: with it, kernels scheduled early waited in pdl_begin() on SMs that
// the copies' completion then had to share, and tsqr_s_host at 4,194,304 x
// 32 took 43.5 ms instead of 5.7 ms.  TSQR wider than 32 columns turns it
// off too: its kernels fill an SM with one CTA, so nothing overlaps, and
// the call at 4,194,304 x 64 was 0.7% slower with it (5.157 against
// 5.122 ms).
inline bool& pdl_allowed() {
    thread_local bool v = true;
    return v;
}
struct PdlOff {
    bool prev;
    explicit PdlOff(bool off = true) : prev(pdl_allowed()) {
        if (off) pdl_allowed() = false;
    }
    ~PdlOff() { pdl_allowed() = prev; }
};

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl_allowed() ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// TMA tensor map of a column-major FP32 matrix (rows x cols, leading
// dimension ld) for boxes of box_rows x box_cols; rows and columns past the
// ends read as zeros.  swizzle128: the 128-byte swizzle (box_rows * 4 must
// then be 128; the destination must be 1024-byte aligned), where the 16-byte
// chunk q of the box's column c lands at chunk q ^ (c % 8).  False when the
// matrix does not meet TMA's rules (16-byte base, ld a multiple of 4 floats)
// or the driver offers no encoder (tsqr.cu).
bool tensor_map_f32(CUtensorMap* map, const float* base, int64_t ld, int64_t rows, int64_t cols, int box_rows,
                    int box_cols, bool swizzle128);

// Streaming multiprocessors of the current device, cached per device (148
// if the attribute cannot be read; the launch that follows then reports the
// error).
inline int device_sm_count() {
    static std::atomic<int> cache[kMaxDevices];
    const int dev = current_device();
    const bool cached = dev >= 0 && dev < kMaxDevices;
    if (cached) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
    if (cached) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

// Polls allowed to the in-loop MMA waits of the tensor-core kernels
// (tc_apply_tiles, tc_gemm_kernel); their clean-up waits before TMEM is
// freed always keep the full limit.  Lowered only by the test entry point
// tsqr_debug_set_wait_limit, to make a wait run out on purpose.
constexpr int kDefaultWaitTries = 1 << 24;
inline std::atomic<int>& wait_tries() {
    static std::atomic<int> v{kDefaultWaitTries};
    return v;
}

// Launch log for the instrumented entry point: when active on this host
// thread, every kernel launch of the library records a CUDA event after it
// on the launch stream, so per-launch device times can be read back.
struct LaunchLog {
    static constexpr int kMax = 512;
    cudaEvent_t ev[kMax + 1];
    int tag[kMax];
    int count = 0;
};
extern thread_local LaunchLog* tl_log;
inline void log_launch(int tag, cudaStream_t s) {
    if (tl_log && tl_log->count < LaunchLog::kMax) {
        tl_log->tag[tl_log->count] = tag;
        cudaEventRecord(tl_log->ev[++tl_log->count], s);
    }
}
// Launch tags: kind * 1000 + level.
enum { kTagFactor = 1000, kTagApply = 2000, kTagGemmTN = 3000, kTagReduce = 4000, kTagGemmNN = 5000,
       kTagAxpy = 6000, kTagTc = 7000, kTagBatched = 8000, kTagApplyQt = 9000, kTagHouse = 10000 };

// Plain-precision TSQR tree (tsqr.cu).  phases: the up-sweep (factor every
// level, R out) and / or the down-sweep (explicit Q from the compact-WY
// tree left in A and the workspace by the up-sweep).
enum { kPhaseUp = 1, kPhaseDown = 2 };
template <typename T>
size_t tsqr_plain_workspace(int64_t m, int64_t n);
template <typename T>
tsqr_status tsqr_plain(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                       cudaStream_t s, int phases = kPhaseUp | kPhaseDown);
// One level of the tree as the up-sweep leaves it: h rows (column-major, ld)
// cut into ntiles tiles of `rows` rows, each holding V below its diagonal
// and T in its top block's upper triangle; level 0 is A, the last level is
// the root.
template <typename T>
struct TreeLevel {
    T* M;
    int64_t ld, h, ntiles;
    int rows;
};
template <typename T>
tsqr_status tsqr_plain_tree(int64_t m, int64_t n, const T* A, int64_t lda, const void* work, size_t work_bytes,
                            std::vector<TreeLevel<T>>* out);

// Recursive blocked QR (blocked_qr.cu).
template <typename T>
size_t qr_workspace(int64_t m, int64_t n, const tsqr_opts& o);
template <typename T>
tsqr_status qr_run(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                   const tsqr_opts& o, cudaStream_t s);

// R <- R2 R of two n x n upper triangular factors (n <= 64 for float, 32
// for double), zeros below the diagonal (tsqr.cu).
template <typename T>
tsqr_status upper_product(int n, const T* R2, int64_t ld2, T* R, int64_t ldr, cudaStream_t s);

// Library-owned per-device buffer for the reference-signature entry points.
void* cached_workspace(size_t bytes, tsqr_status* st);

}  // namespace tsqr

namespace tsqr {
// Precision form of TSQR (tsqr.cu + tc_apply.cu), FP32 only.  Options:
// norm64 -- per-column norm, beta and tau in FP64 (tsqr_opts.fp64_scalars);
// root64 -- root combine in FP64, n <= 32 (tsqr_opts.fp64_root);
// clear_status -- zero the status word first (off for a second pass that
// must keep the first pass's report).
struct PrecFlags {
    bool norm64 = false;
    bool root64 = false;
    bool clear_status = true;
};
size_t tsqr_precision_workspace(int64_t m, int64_t n, PrecFlags f = PrecFlags());
// TSQR of host-resident A with host Q and R, transfers pipelined with the
// level-0 kernels (tsqr.cu).  prec: the precision form (FP32 only).
template <typename T>
size_t tsqr_host_workspace(int64_t m, int64_t n, bool prec);
template <typename T>
tsqr_status tsqr_host(int64_t m, int64_t n, const T* hA, int64_t lda, T* hQ, int64_t ldq, T* hR, int64_t ldr,
                      void* work, size_t work_bytes, bool prec, cudaStream_t s);
tsqr_status tsqr_precision(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                           size_t work_bytes, cudaStream_t s, PrecFlags f = PrecFlags());
}  // namespace tsqr

namespace tsqr {
// tcgen05 GEMMs of the blocked QR precision forms (tc_gemm.cu): TF32x3, or
// BF16x3 with bf16 = true.
int tc_tn_splits(int64_t M, int64_t N, int64_t K);
int tc_gemm_tn(int M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb, float* P, int* err,
               cudaStream_t s, bool bf16 = false);
void tc_gemm_nn(int64_t M, int N, int K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
                float* C, int64_t ldc, int* err, cudaStream_t s, bool bf16 = false);
}  // namespace tsqr

namespace tsqr {
// Batched TSQR (batched.cu), FP32, n <= 64.
size_t batched_workspace(int count, const int64_t* m, const int64_t* n);
tsqr_status batched_tune(int count, const int64_t* m, const int64_t* n, int reps, cudaStream_t s);
int batched_choice(int width_class, int height_bucket);
int batched_candidate_rows(int width_class, int candidate);
tsqr_status batched_set_choice(int width_class, int height_bucket, int candidate);
tsqr_status batched_run(int count, float* const* A, const int64_t* m, const int64_t* n, const int64_t* lda,
                        float* const* R, const int64_t* ldr, void* work, size_t work_bytes, cudaStream_t s);
}  // namespace tsqr
