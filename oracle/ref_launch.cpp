// ref_launch.cpp -- host launcher for the reference's own CUDA kernels.
//
// TEST INFRASTRUCTURE ONLY (golden-vector generation and the reference-side
// timing).  The kernels come from oracle/_ref/ref_kernels.cubin, which
// build_oracle.py compiles unmodified from the reference checkout.  This file
// contains no reference source: it restates the reference host schedules,
//   tsqr<T>  TallShinnyQR.h:86-148   (1-launch case or 2 tsqr_kernel launches
//                                     + tsgemm_tsqr fix-up)
//   qr<T>    block_QR.h:72-95        (recursive block Gram-Schmidt)
// and launches the cubin's kernels through the CUDA driver API (dlopen'd, so
// no link-time dependency on libcuda).
//
// The reference kernels are compiled with NUM_SM=108, BLOCK_SIZE=128,
// BLOCK_DIM_X=32, BLOCK_DIM_Y=16 (kernelQR.h:3-8) and N_B=32 (block_QR.h:5);
// the schedule below must use the same constants.
//
// Safety: the reference's tsqr_kernel spins on a global counter without a
// bound (kernelQR.h:374-375, :426-439, :462, :482) and assumes every CTA is
// resident at once; its per-thread arrays hold n <= 32 columns
// (kernelQR.h:7, :80).  Every entry point checks, before any launch, that
// the launch has at most NUM_SM=108 CTAs (fewer than the GPU's SMs, checked
// against the device), that n <= 32 with BLOCK_SIZE % n == 0, the size
// guards of TallShinnyQR.h:92-109,129, and that the shared-memory level count
// the reference computes (TallShinnyQR.h:111-114, :131-139) covers the
// levels the kernel will actually walk.  Anything else is refused.
#include <cuda.h>
#include <dlfcn.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace {

constexpr int kNumSm = 108;
constexpr int kBlock = 128;
constexpr int kNb = 32;

struct Api {
    void* h = nullptr;
    CUresult (*cuInit)(unsigned);
    CUresult (*cuCtxGetCurrent)(CUcontext*);
    CUresult (*cuDeviceGet)(CUdevice*, int);
    CUresult (*cuDevicePrimaryCtxRetain)(CUcontext*, CUdevice);
    CUresult (*cuCtxSetCurrent)(CUcontext);
    CUresult (*cuCtxGetDevice)(CUdevice*);
    CUresult (*cuDeviceGetAttribute)(int*, CUdevice_attribute, CUdevice);
    CUresult (*cuModuleLoad)(CUmodule*, const char*);
    CUresult (*cuModuleGetFunction)(CUfunction*, CUmodule, const char*);
    CUresult (*cuFuncSetAttribute)(CUfunction, CUfunction_attribute, int);
    CUresult (*cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                               unsigned, CUstream, void**, void**);
} api;

CUmodule g_mod = nullptr;
CUfunction f_tsqr[2], f_tsgemm[2], f_gemm[2];  // [0] float, [1] double
int g_sm_count = 0;

template <typename F>
bool sym(F& fp, const char* name) {
    fp = reinterpret_cast<F>(dlsym(api.h, name));
    return fp != nullptr;
}

// Itanium-ABI names of the explicit instantiations at kernelQR.h:498-507,
// TallShinnyQR.h:75-84 and block_QR.h:61-70.
const char* kTsqrName[2] = {"_Z11tsqr_kernelIfEviiiPT_iS1_iS1_i", "_Z11tsqr_kernelIdEviiiPT_iS1_iS1_i"};
const char* kTsgemmName[2] = {"_Z11tsgemm_tsqrIfEviiiiT_PS0_iS1_iS0_S1_i",
                              "_Z11tsgemm_tsqrIdEviiiiT_PS0_iS1_iS0_S1_i"};
const char* kGemmName[2] = {"_Z12gemm_blockqrIfEviiiT_iPS0_iS1_iS0_S1_i",
                            "_Z12gemm_blockqrIdEviiiT_iPS0_iS1_iS0_S1_i"};

// Number of up-sweep levels tsqr_kernel walks on a chunk of height h
// (kernelQR.h:341-388).
int walk_levels(int h, int n) {
    int levels = 0;
    while (h > n || levels == 0) {
        ++levels;
        h = ((h + kBlock - 1) / kBlock) * n;
    }
    return levels;
}

template <typename T>
int launch_tsqr_kernel(int which, int grid, int m_total, int m_each, int n, T* A, int lda, T* R, int ldr,
                       T* work, int ldwork, int smem, CUstream s) {
    void* args[] = {&m_total, &m_each, &n, &A, &lda, &R, &ldr, &work, &ldwork};
    return (int)api.cuLaunchKernel(f_tsqr[which], grid, 1, 1, 32, 16, 1, smem, s, args, nullptr);
}

// tsqr<T> host schedule (TallShinnyQR.h:86-148).
template <typename T>
int ref_tsqr(int which, int m, int n, T* A, int lda, T* R, int ldr, T* work, int ldwork, CUstream s) {
    if (!g_mod) return 100;
    if (m < n || n < 1 || n > 32 || kBlock % n != 0) return 101;  // :92-93 and kernelQR.h:7
    if (ldwork < 2 * kNumSm * kBlock) return 102;                 // work layout of :90
    if (g_sm_count < kNumSm) return 103;                          // co-residency of 108 CTAs
    const int max_grid = kNumSm * kBlock;
    if ((long long)m > (long long)(max_grid / n) * max_grid) return 104;  // :100-103
    const int grid_num = (m + max_grid - 1) / max_grid;
    T* work1 = work;
    T* work2 = work + max_grid;
    if (grid_num > 1) {
        if ((m % max_grid) % n != 0) return 105;  // :109
        int rt = (int)std::ceil((std::log((double)max_grid) - std::log((double)n)) /
                                (std::log((double)kBlock) - std::log((double)n)));
        int need = walk_levels(max_grid, n);
        int last = m % max_grid;
        if (last && walk_levels(last, n) > need) need = walk_levels(last, n);
        if (walk_levels(grid_num * n, n) > need) need = walk_levels(grid_num * n, n);
        if (need > rt) return 106;
        int smem = rt * kBlock * n * (int)sizeof(T);
        int rc = (int)api.cuFuncSetAttribute(f_tsqr[which], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem);
        if (rc) return rc;
        rc = launch_tsqr_kernel<T>(which, kNumSm, m, max_grid, n, A, lda, work1, ldwork, work2, ldwork, smem, s);
        if (rc) return rc;
        rc = launch_tsqr_kernel<T>(which, kNumSm, grid_num * n, grid_num * n, n, work1, ldwork, R, ldr, work2,
                                   ldwork, smem, s);
        if (rc) return rc;
        int m_total = m, m_each = max_grid, nn = n, k = n;
        T alpha = 1, beta = 0;
        void* args[] = {&m_total, &m_each, &nn, &k, &alpha, &A, &lda, &work1, &ldwork, &beta, &A, &lda};
        return (int)api.cuLaunchKernel(f_tsgemm[which], kNumSm, 1, 1, 32, 32, 1, 0, s, args, nullptr);
    }
    if ((m % kBlock) % n != 0) return 105;  // :129
    int rt = (m == n) ? 1
                      : (int)std::ceil((std::log((double)m) - std::log((double)n)) /
                                       (std::log((double)kBlock) - std::log((double)n)));
    if (walk_levels(m, n) > rt) return 106;
    int smem = rt * kBlock * n * (int)sizeof(T);
    int rc = (int)api.cuFuncSetAttribute(f_tsqr[which], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem);
    if (rc) return rc;
    int blocks = (m + kBlock - 1) / kBlock;
    return launch_tsqr_kernel<T>(which, blocks, m, m, n, A, lda, R, ldr, work2, ldwork, smem, s);
}

// qr<T> host schedule (block_QR.h:72-95).
template <typename T>
int ref_qr(int which, int m, int n, T* A, int lda, T* R, int ldr, T* work, int ldwork, CUstream s) {
    if (n <= kNb) return ref_tsqr<T>(which, m, n, A, lda, R, ldr, work, ldwork, s);
    if (n % 2 != 0 || (n / 2) % kNb != 0) return 101;  // block_QR.h:78-79
    int n1 = n / 2;
    T* A1 = A;
    T* A2 = A + (size_t)n1 * lda;
    T* R11 = R;
    T* R12 = R + (size_t)n1 * ldr;
    T* R22 = R + (size_t)n1 * ldr + n1;
    int rc = ref_qr<T>(which, m, n1, A1, lda, R11, ldr, work, ldwork, s);
    if (rc) return rc;
    unsigned g1 = (unsigned)((n1 + 31) / 32);
    {
        int mm = n1, nn = n1, k = m, trans = 1;
        T alpha = 1, beta = 0;
        void* args[] = {&mm, &nn, &k, &alpha, &trans, &A1, &lda, &A2, &lda, &beta, &R12, &ldr};
        rc = (int)api.cuLaunchKernel(f_gemm[which], g1, g1, 1, 32, 32, 1, 0, s, args, nullptr);
        if (rc) return rc;
    }
    {
        int mm = m, nn = n1, k = n1, trans = 0;
        T alpha = -1, beta = 1;
        void* args[] = {&mm, &nn, &k, &alpha, &trans, &A1, &lda, &R12, &ldr, &beta, &A2, &lda};
        rc = (int)api.cuLaunchKernel(f_gemm[which], kNumSm, 1, 1, 32, 32, 1, 0, s, args, nullptr);
        if (rc) return rc;
    }
    return ref_qr<T>(which, m, n1, A2, lda, R22, ldr, work, ldwork, s);
}

}  // namespace

extern "C" {

// Loads the cubin into the current (or the primary) context of device 0.
// Returns 0 on success.
int refl_init(const char* cubin_path) {
    if (g_mod) return 0;
    api.h = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!api.h) return 1;
    if (!sym(api.cuInit, "cuInit") || !sym(api.cuCtxGetCurrent, "cuCtxGetCurrent") ||
        !sym(api.cuDeviceGet, "cuDeviceGet") || !sym(api.cuDevicePrimaryCtxRetain, "cuDevicePrimaryCtxRetain") ||
        !sym(api.cuCtxSetCurrent, "cuCtxSetCurrent") || !sym(api.cuCtxGetDevice, "cuCtxGetDevice") ||
        !sym(api.cuDeviceGetAttribute, "cuDeviceGetAttribute") || !sym(api.cuModuleLoad, "cuModuleLoad") ||
        !sym(api.cuModuleGetFunction, "cuModuleGetFunction") ||
        !sym(api.cuFuncSetAttribute, "cuFuncSetAttribute") || !sym(api.cuLaunchKernel, "cuLaunchKernel"))
        return 2;
    if (api.cuInit(0)) return 3;
    CUcontext ctx = nullptr;
    api.cuCtxGetCurrent(&ctx);
    if (!ctx) {
        CUdevice dev;
        if (api.cuDeviceGet(&dev, 0)) return 4;
        if (api.cuDevicePrimaryCtxRetain(&ctx, dev)) return 5;
        if (api.cuCtxSetCurrent(ctx)) return 6;
    }
    CUdevice dev;
    if (api.cuCtxGetDevice(&dev)) return 7;
    if (api.cuDeviceGetAttribute(&g_sm_count, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev)) return 8;
    CUmodule mod;
    if (api.cuModuleLoad(&mod, cubin_path)) return 9;
    for (int w = 0; w < 2; ++w) {
        if (api.cuModuleGetFunction(&f_tsqr[w], mod, kTsqrName[w])) return 10;
        if (api.cuModuleGetFunction(&f_tsgemm[w], mod, kTsgemmName[w])) return 11;
        if (api.cuModuleGetFunction(&f_gemm[w], mod, kGemmName[w])) return 12;
    }
    g_mod = mod;
    return 0;
}

// Work buffers follow the reference drivers: ldwork >= 2*NUM_SM*BLOCK_SIZE
// (27648) rows, ldwork*n elements (test_tsqr.cu:42-45).  All pointers are
// device pointers.  Launches go to `stream` (the reference uses stream 0).
int refl_tsqr_f(int m, int n, float* A, int lda, float* R, int ldr, float* work, int ldwork, void* stream) {
    return ref_tsqr<float>(0, m, n, A, lda, R, ldr, work, ldwork, (CUstream)stream);
}
int refl_tsqr_d(int m, int n, double* A, int lda, double* R, int ldr, double* work, int ldwork, void* stream) {
    return ref_tsqr<double>(1, m, n, A, lda, R, ldr, work, ldwork, (CUstream)stream);
}
int refl_qr_f(int m, int n, float* A, int lda, float* R, int ldr, float* work, int ldwork, void* stream) {
    return ref_qr<float>(0, m, n, A, lda, R, ldr, work, ldwork, (CUstream)stream);
}
int refl_qr_d(int m, int n, double* A, int lda, double* R, int ldr, double* work, int ldwork, void* stream) {
    return ref_qr<double>(1, m, n, A, lda, R, ldr, work, ldwork, (CUstream)stream);
}
int refl_ldwork(void) { return 2 * kNumSm * kBlock; }

}  // extern "C"
