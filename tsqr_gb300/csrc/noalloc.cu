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
//     cudaGetSymbolAddress, taken once per device, with that device
//     current, on the first call made on the device.  Make that first call
//     before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tsqr_gb300.h"
#include "internal.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[TSQR_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device (set-up on the
// first call per device).
tsqr_status scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TSQR_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_scratch_ptr[dev] == nullptr) {
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
    tsqr_status st = scratch_address(&scratch);
    if (st != TSQR_OK) return st;
    return tsqr::tsqr_plain<float>(m, n, A, lda, R, ldr, scratch, (size_t)TSQR_NOALLOC_SCRATCH_BYTES,
                                   (cudaStream_t)stream);
}
