// noalloc.cu -- FP32 TSQR for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at all.  Some run inside frameworks that
// have already reserved nearly all device memory for their own pool, so an
// extra allocation fails or fragments that pool.  Others work to a memory
// budget set at start-up, or cannot afford the device-wide synchronisation
// that cudaFree may cause.  Others call through the reference's interface,
// whose d_work was sized for the reference's layout and cannot grow.
// tsqr_s_noalloc serves them: it runs the same plain FP32 TSQR tree as
// tsqr_s_ex, but its tree workspace (the stacked R factors of the upper
// levels) lives in one file-scope __device__ array of
// TSQR_NOALLOC_SCRATCH_BYTES, so the call itself allocates nothing.
//
// Rules of the array:
//   * every GPU that loads this library holds the array until the process
//     exits;
//   * all calls on a device share it and leave their data in it, so calls
//     whose work overlaps on the GPU (different streams, or host threads
//     without ordering) race with each other and must be serialised by the
//     caller;
//   * nothing in it needs to start at zero: every byte a call reads was
//     written earlier in the same call;
//   * host code may not use the array's name as a device address (on the
//     host it names a stand-in); the device address comes from
//     cudaGetSymbolAddress, with the device current.  The first call made on
//     a device takes it (this may load the library's device code), so make
//     that first call before any stream capture.  Later calls look it up
//     again whenever their stream is not capturing -- after a
//     cudaDeviceReset the array may sit at a new address -- and a call on a
//     capturing stream uses the address of the last such lookup.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tsqr_gb300.h"
#include "internal.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TSQR_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device: looked up
// when the call's stream is not capturing (and on the first call of the
// device), otherwise the last address looked up.
tsqr_status scratch_address(cudaStream_t s, void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TSQR_ERR_NO_DEVICE;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const bool query_failed = cudaStreamIsCapturing(s, &cap) != cudaSuccess;
    if (query_failed) (void)cudaGetLastError();  // the failed query's own error only
    const bool capturing = query_failed || cap != cudaStreamCaptureStatusNone;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_scratch_ptr[dev] == nullptr || !capturing) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return TSQR_ERR_CUDA;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return TSQR_OK;
}

}  // namespace

extern "C" tsqr_status tsqr_s_noalloc(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr,
                                      void* stream) {
    if (m < 1 || n < 1 || m < n || lda < m || ldr < n || A == nullptr || R == nullptr) return TSQR_ERR_INVALID_ARG;
    if (n > 64) return TSQR_ERR_UNSUPPORTED;
    const size_t need = tsqr::tsqr_plain_workspace<float>(m, n);
    if (need == 0) return TSQR_ERR_UNSUPPORTED;
    if (need > (size_t)TSQR_NOALLOC_SCRATCH_BYTES) return TSQR_ERR_WORKSPACE;
    void* scratch = nullptr;
    tsqr_status st = scratch_address((cudaStream_t)stream, &scratch);
    if (st != TSQR_OK) return st;
    return tsqr::tsqr_plain<float>(m, n, A, lda, R, ldr, scratch, (size_t)TSQR_NOALLOC_SCRATCH_BYTES,
                                   (cudaStream_t)stream);
}
