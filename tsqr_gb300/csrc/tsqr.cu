// tsqr.cu -- TSQR host driver and C ABI entry points (plain precision path).
//
// Replaces the reference host driver tsqr<T> (TallShinnyQR.h:86-148).  The
// reference picks between a single persistent launch (m <= NUM_SM*BLOCK_SIZE)
// and a chunk loop + second TSQR + fix-up GEMM; here one reduction tree of
// runtime height covers every m: one factor launch per level going up, one
// apply launch per level coming down, all on the caller's stream, with no
// grid-wide spin barrier (kernelQR.h:297, :374) and no global state, so
// concurrent calls on different streams with different workspaces are safe.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/tsqr_gb300.h"
#include "internal.h"
#include "tsqr_kernels.cuh"

namespace tsqr {

thread_local LaunchLog* tl_log = nullptr;

namespace {

template <typename T, int NMAX, int NT, int RPT, int MINB, int AMINB, bool NORM64 = false>
struct TileCfg {
    static constexpr int kRows = NT * RPT;
    static void factor(const FactorParams<T>& p, int grid, cudaStream_t s) {
        factor_tiles<T, NMAX, NT, RPT, MINB, NORM64><<<grid, NT, 0, s>>>(p);
    }
    static void apply(const ApplyParams<T>& p, int grid, cudaStream_t s) {
        constexpr size_t smem = apply_smem_bytes<T, NMAX>();
        static bool attr = [] {
            return cudaFuncSetAttribute(apply_tiles<T, NMAX, NT, RPT, AMINB>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
        }();
        (void)attr;
        apply_tiles<T, NMAX, NT, RPT, AMINB><<<grid, NT, smem, s>>>(p);
    }
};

template <typename T>
struct KernelSet {
    int rows = 0;  // tile height B
    void (*factor)(const FactorParams<T>&, int, cudaStream_t) = nullptr;
    void (*apply)(const ApplyParams<T>&, int, cudaStream_t) = nullptr;
};

template <typename C, typename T>
KernelSet<T> make_set() {
    KernelSet<T> k;
    k.rows = C::kRows;
    k.factor = &C::factor;
    k.apply = &C::apply;
    return k;
}

// Tile configuration per (dtype, n).  The tile height B is the tree arity
// times n; B >= 4n keeps the stacked-R levels at most a quarter of the level
// below, and the tile stays in registers (RPT rows x NMAX columns/thread).
KernelSet<float> pick(float*, int n) {
    if (n <= 8) return make_set<TileCfg<float, 8, 256, 4, 3, 3>, float>();
    if (n <= 16) return make_set<TileCfg<float, 16, 256, 2, 2, 3>, float>();
    if (n <= 32) return make_set<TileCfg<float, 32, 256, 2, 2, 1>, float>();
    if (n <= 64) return make_set<TileCfg<float, 64, 256, 1, 1, 1>, float>();
    return KernelSet<float>();
}
KernelSet<double> pick(double*, int n) {
    if (n <= 8) return make_set<TileCfg<double, 8, 256, 2, 2, 3>, double>();
    if (n <= 16) return make_set<TileCfg<double, 16, 256, 2, 1, 2>, double>();
    if (n <= 32) return make_set<TileCfg<double, 32, 256, 1, 1, 1>, double>();
    return KernelSet<double>();
}

template <typename T>
struct Level {
    T* M;
    int64_t ld;
    int64_t h;
    int64_t ntiles;
};

constexpr size_t kAlign = 256;

// Lays the tree out in the workspace.  With base == nullptr only the size is
// computed.  Returns the bytes used.
template <typename T>
size_t plan_levels(int64_t m, int64_t n, T* A, int64_t lda, int rows, char* base, std::vector<Level<T>>* out) {
    size_t off = 0;
    std::vector<Level<T>> lv;
    lv.push_back({A, lda, m, ceil_div(m, rows)});
    while (lv.back().ntiles > 1) {
        const int64_t h = lv.back().ntiles * n;
        const int64_t ld = round_up(h, 32);
        T* M = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += (size_t)round_up((int64_t)(ld * n * (int64_t)sizeof(T)), (int64_t)kAlign);
        lv.push_back({M, ld, h, ceil_div(h, rows)});
    }
    if (out) *out = lv;
    return off;
}

}  // namespace

template <typename T>
size_t tsqr_plain_workspace(int64_t m, int64_t n) {
    KernelSet<T> ks = pick((T*)nullptr, (int)n);
    if (!ks.factor) return 0;
    size_t b = plan_levels<T>(m, n, nullptr, m, ks.rows, nullptr, nullptr);
    return b ? b : kAlign;  // never report 0 for a valid size
}

template <typename T>
tsqr_status tsqr_plain(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                       cudaStream_t s) {
    KernelSet<T> ks = pick((T*)nullptr, (int)n);
    if (!ks.factor) return TSQR_ERR_UNSUPPORTED;
    std::vector<Level<T>> lv;
    size_t need = plan_levels<T>(m, n, A, lda, ks.rows, reinterpret_cast<char*>(work), &lv);
    if (need > 0 && (work == nullptr || work_bytes < need)) return TSQR_ERR_WORKSPACE;
    const int L = (int)lv.size();
    // up-sweep
    for (int l = 0; l < L; ++l) {
        FactorParams<T> fp;
        fp.M = lv[l].M;
        fp.ld = lv[l].ld;
        fp.h = lv[l].h;
        fp.n = (int)n;
        fp.ntiles = lv[l].ntiles;
        if (l == L - 1) {
            fp.Rout = R;
            fp.ldr = ldr;
        } else {
            fp.Rout = lv[l + 1].M;
            fp.ldr = lv[l + 1].ld;
        }
        ks.factor(fp, (int)std::min<int64_t>(lv[l].ntiles, 1 << 30), s);
        log_launch(kTagFactor + l, s);
    }
    // down-sweep
    for (int l = L - 1; l >= 0; --l) {
        ApplyParams<T> ap;
        ap.M = lv[l].M;
        ap.ld = lv[l].ld;
        ap.h = lv[l].h;
        ap.n = (int)n;
        ap.ntiles = lv[l].ntiles;
        ap.P = (l == L - 1) ? nullptr : lv[l + 1].M;
        ap.ldp = (l == L - 1) ? 0 : lv[l + 1].ld;
        ks.apply(ap, (int)std::min<int64_t>(lv[l].ntiles, 1 << 30), s);
        log_launch(kTagApply + l, s);
    }
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

template size_t tsqr_plain_workspace<float>(int64_t, int64_t);
template size_t tsqr_plain_workspace<double>(int64_t, int64_t);
template tsqr_status tsqr_plain<float>(int64_t, int64_t, float*, int64_t, float*, int64_t, void*, size_t,
                                       cudaStream_t);
template tsqr_status tsqr_plain<double>(int64_t, int64_t, double*, int64_t, double*, int64_t, void*, size_t,
                                        cudaStream_t);

// ---------------------------------------------------------------------------
// Per-device workspace cache for the reference-signature entry points, whose
// d_work is sized for the reference's own layout (ldwork*n elements with
// ldwork = 2*NUM_SM*BLOCK_SIZE, test_tsqr.cu:42-45).
// ---------------------------------------------------------------------------
void* cached_workspace(size_t bytes, tsqr_status* st) {
    static std::mutex mu;
    static void* buf[64] = {nullptr};
    static size_t cap[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        *st = TSQR_ERR_NO_DEVICE;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (cap[dev] < bytes) {
        if (buf[dev]) {
            cudaDeviceSynchronize();
            cudaFree(buf[dev]);
            buf[dev] = nullptr;
            cap[dev] = 0;
        }
        if (cudaMalloc(&buf[dev], bytes) != cudaSuccess) {
            buf[dev] = nullptr;
            *st = TSQR_ERR_CUDA;
            return nullptr;
        }
        cap[dev] = bytes;
    }
    *st = TSQR_OK;
    return buf[dev];
}

}  // namespace tsqr
