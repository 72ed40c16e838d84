// batched.cu -- many independent FP32 TSQR problems of uneven heights and
// widths (n <= 64) in one short sequence of launches.  No counterpart in the
// reference, which factors one matrix per call (TallShinnyQR.h:86).
//
// Every problem keeps its own reduction tree, laid out in the workspace
// exactly as the single-problem path lays it out.  Problems are grouped by
// width class (n <= 8, 16, 32, 64: the register-tile configuration of the
// single-problem path).  For each class the up-sweep is one launch per tree
// level covering the tiles of every problem of the class that has that
// level, and the down-sweep one launch per level in reverse.  A launch's
// work list is a table of per-problem descriptors (level matrix, its height
// and leading dimension, where its R factors go or which parent block it
// multiplies by, and the index of its first tile in the launch's global tile
// numbering), passed by value in the kernel parameter space: the call
// performs no host-to-device copy and no allocation, so it can be captured
// into a CUDA graph and replayed as one launch.  CTAs are persistent
// (grid = SMs x resident CTAs) and find the problem of each global tile by
// binary search in the table.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "internal.h"
#include "tsqr_kernels.cuh"

namespace tsqr {

namespace {

constexpr int kTable = 448;  // descriptors per launch (fits the 32 KB parameter space)

struct FactorItem {
    float* M;
    float* Rout;
    int64_t ld;
    int64_t ldr;
    int h;
    int n;
    int64_t tile0;  // first global tile index of this problem in the launch
};
struct FactorTable {
    int count;
    int64_t total;  // tiles in the launch
    FactorItem it[kTable];
};

struct ApplyItem {
    float* M;
    const float* P;  // parent level (rows t*n of tile t); null = identity
    int64_t ld;
    int64_t ldp;
    int h;
    int n;
    int64_t tile0;
};
struct ApplyTable {
    int count;
    int64_t total;
    ApplyItem it[kTable];
};

template <typename Item>
__device__ __forceinline__ int find_item(const Item* it, int count, int64_t t) {
    int lo = 0, hi = count - 1;
    while (lo < hi) {  // last item with tile0 <= t
        const int mid = (lo + hi + 1) >> 1;
        if (it[mid].tile0 <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

template <int NMAX, int NT, int RPT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batched_factor(const __grid_constant__ FactorTable tab) {
    constexpr int B = NT * RPT;
    __shared__ FactorSmem<float, NMAX, NT, false> S;
    for (int64_t t = blockIdx.x; t < tab.total; t += gridDim.x) {
        const int i = find_item(tab.it, tab.count, t);
        const FactorItem& w = tab.it[i];
        const int64_t lt = t - w.tile0;
        const int64_t row0 = lt * B;
        const int ht = (int)((w.h - row0) < B ? (w.h - row0) : B);
        factor_tile<float, NMAX, NT, RPT, false>(S, w.M + row0, w.ld, ht, w.n, w.Rout + lt * w.n, w.ldr);
    }
}

template <int NMAX, int CW, int RPT, int MINB>
__global__ void __launch_bounds__(32 * (NMAX / CW), MINB) batched_factor_split(const __grid_constant__ FactorTable tab) {
    constexpr int B = 32 * RPT;
    __shared__ SplitFactorSmem<float, NMAX, CW, RPT> S;
    for (int64_t t = blockIdx.x; t < tab.total; t += gridDim.x) {
        const int i = find_item(tab.it, tab.count, t);
        const FactorItem& w = tab.it[i];
        const int64_t lt = t - w.tile0;
        const int64_t row0 = lt * B;
        const int ht = (int)((w.h - row0) < B ? (w.h - row0) : B);
        factor_split_tile<float, NMAX, CW, RPT, false>(S, w.M + row0, w.ld, ht, w.n, w.Rout + lt * w.n, w.ldr);
    }
}

template <int NMAX, int NT, int RPT, int MINB>
__global__ void __launch_bounds__(NT, MINB) batched_apply(const __grid_constant__ ApplyTable tab) {
    constexpr int B = NT * RPT;
    extern __shared__ __align__(16) unsigned char apply_smem[];
    for (int64_t t = blockIdx.x; t < tab.total; t += gridDim.x) {
        const int i = find_item(tab.it, tab.count, t);
        const ApplyItem& w = tab.it[i];
        const int64_t lt = t - w.tile0;
        const int64_t row0 = lt * B;
        const int ht = (int)((w.h - row0) < B ? (w.h - row0) : B);
        const float* Pb = w.P ? w.P + lt * w.n : nullptr;
        apply_tile<float, NMAX, NT, RPT>(apply_smem, w.M + row0, w.ld, ht, w.n, Pb, w.ldp, 0);
    }
}

// Per-class configuration; tile heights and kernels equal those of the
// single-problem path (tsqr.cu), so a problem's tree and arithmetic are the
// same either way.
struct ClassCfg {
    int nmax, rows;
    int factor_per_sm, apply_per_sm;  // resident CTAs per SM of each kernel
    void (*factor)(const FactorTable&, int, cudaStream_t);
    void (*apply)(const ApplyTable&, int, cudaStream_t);
};

template <int NMAX, int B, int ANT, int AMINB>
void class_apply(const ApplyTable& t, int grid, cudaStream_t s) {
    constexpr int ARPT = B / ANT;  // the apply CTA covers the tile height
    constexpr size_t kSmem = apply_smem_bytes<float, NMAX, B>();
    static bool attr = [] {
        return cudaFuncSetAttribute(batched_apply<NMAX, ANT, ARPT, AMINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmem) == cudaSuccess;
    }();
    (void)attr;
    batched_apply<NMAX, ANT, ARPT, AMINB><<<grid, ANT, kSmem, s>>>(t);
}

// one thread per row slice (factor_tile)
template <int NMAX, int NT, int RPT, int MINB, int AMINB, int ANT = NT>
struct Cls {
    static void factor(const FactorTable& t, int grid, cudaStream_t s) {
        batched_factor<NMAX, NT, RPT, MINB><<<grid, NT, 0, s>>>(t);
    }
    static ClassCfg cfg() { return {NMAX, NT * RPT, MINB, AMINB, &factor, &class_apply<NMAX, NT * RPT, ANT, AMINB>}; }
};

// column-split tiles (factor_split_tile)
template <int NMAX, int CW, int RPT, int MINB, int AMINB, int ANT>
struct SplitCls {
    static void factor(const FactorTable& t, int grid, cudaStream_t s) {
        batched_factor_split<NMAX, CW, RPT, MINB><<<grid, 32 * (NMAX / CW), 0, s>>>(t);
    }
    static ClassCfg cfg() { return {NMAX, 32 * RPT, MINB, AMINB, &factor, &class_apply<NMAX, 32 * RPT, ANT, AMINB>}; }
};

const ClassCfg& class_of(int n) {
    static const ClassCfg c8 = Cls<8, 256, 4, 3, 3>::cfg();
    static const ClassCfg c16 = SplitCls<16, 4, 16, 4, 3, 256>::cfg();
    static const ClassCfg c32 = SplitCls<32, 4, 16, 2, 2, 256>::cfg();
    static const ClassCfg c64 = SplitCls<64, 8, 16, 1, 1, 256>::cfg();
    if (n <= 8) return c8;
    if (n <= 16) return c16;
    if (n <= 32) return c32;
    return c64;
}

struct Lvl {
    float* M;
    int64_t ld, h, ntiles;
};

// The problem's tree inside its workspace block (same layout rule as
// plan_levels in tsqr.cu).
size_t tree_of(int64_t m, int64_t n, float* A, int64_t lda, int rows, char* base, std::vector<Lvl>* out) {
    size_t off = 0;
    std::vector<Lvl> lv;
    lv.push_back({A, lda, m, ceil_div(m, rows)});
    while (lv.back().ntiles > 1) {
        const int64_t h = lv.back().ntiles * n;
        const int64_t ld = round_up(h, 32);
        float* M = base ? reinterpret_cast<float*>(base + off) : nullptr;
        off += (size_t)round_up(ld * n * 4, 256);
        lv.push_back({M, ld, h, ceil_div(h, rows)});
    }
    if (out) *out = lv;
    return off < 256 ? 256 : off;
}

int resident_grid(const ClassCfg& c, bool apply, int64_t tiles) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    const int per_sm = apply ? c.apply_per_sm : c.factor_per_sm;
    return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sms * per_sm));
}

}  // namespace

size_t batched_workspace(int count, const int64_t* m, const int64_t* n) {
    size_t total = 0;
    for (int i = 0; i < count; ++i) {
        if (m[i] < 1 || n[i] < 1 || n[i] > 64 || m[i] < n[i]) return 0;
        total += tree_of(m[i], n[i], nullptr, m[i], class_of((int)n[i]).rows, nullptr, nullptr);
    }
    return total < 256 ? 256 : total;
}

tsqr_status batched_run(int count, float* const* A, const int64_t* m, const int64_t* n, const int64_t* lda,
                        float* const* R, const int64_t* ldr, void* work, size_t work_bytes, cudaStream_t s) {
    if (count == 0) return TSQR_OK;
    const size_t need = batched_workspace(count, m, n);
    if (need == 0) return TSQR_ERR_INVALID_ARG;
    if (work == nullptr || work_bytes < need) return TSQR_ERR_WORKSPACE;
    // Trees of every problem.
    std::vector<std::vector<Lvl>> trees(count);
    char* base = reinterpret_cast<char*>(work);
    size_t off = 0;
    for (int i = 0; i < count; ++i)
        off += tree_of(m[i], n[i], A[i], lda[i], class_of((int)n[i]).rows, base + off, &trees[i]);

    const int classes[4] = {8, 16, 32, 64};
    FactorTable* ft = new FactorTable;
    ApplyTable* at = new ApplyTable;
    tsqr_status st = TSQR_OK;
    for (int ci = 0; ci < 4 && st == TSQR_OK; ++ci) {
        std::vector<int> members;
        for (int i = 0; i < count; ++i)
            if (class_of((int)n[i]).nmax == classes[ci]) members.push_back(i);
        if (members.empty()) continue;
        const ClassCfg& C = class_of(classes[ci]);
        int maxL = 0;
        for (int i : members) maxL = std::max(maxL, (int)trees[i].size());
        // up-sweep: one launch per level (and per table of kTable problems)
        for (int l = 0; l < maxL; ++l) {
            size_t k = 0;
            while (k < members.size()) {
                ft->count = 0;
                ft->total = 0;
                for (; k < members.size() && ft->count < kTable; ++k) {
                    const int i = members[k];
                    const auto& tr = trees[i];
                    if (l >= (int)tr.size()) continue;
                    FactorItem& w = ft->it[ft->count++];
                    w.M = tr[l].M;
                    w.ld = tr[l].ld;
                    w.h = (int)tr[l].h;
                    w.n = (int)n[i];
                    const bool last = (l == (int)tr.size() - 1);
                    w.Rout = last ? R[i] : tr[l + 1].M;
                    w.ldr = last ? ldr[i] : tr[l + 1].ld;
                    w.tile0 = ft->total;
                    ft->total += tr[l].ntiles;
                }
                if (ft->count == 0) continue;
                C.factor(*ft, resident_grid(C, false, ft->total), s);
                log_launch(kTagBatched + l, s);
            }
        }
        // down-sweep
        for (int l = maxL - 1; l >= 0; --l) {
            size_t k = 0;
            while (k < members.size()) {
                at->count = 0;
                at->total = 0;
                for (; k < members.size() && at->count < kTable; ++k) {
                    const int i = members[k];
                    const auto& tr = trees[i];
                    if (l >= (int)tr.size()) continue;
                    ApplyItem& w = at->it[at->count++];
                    w.M = tr[l].M;
                    w.ld = tr[l].ld;
                    w.h = (int)tr[l].h;
                    w.n = (int)n[i];
                    const bool top = (l == (int)tr.size() - 1);
                    w.P = top ? nullptr : tr[l + 1].M;
                    w.ldp = top ? 0 : tr[l + 1].ld;
                    w.tile0 = at->total;
                    at->total += tr[l].ntiles;
                }
                if (at->count == 0) continue;
                C.apply(*at, resident_grid(C, true, at->total), s);
                log_launch(kTagBatched + 500 + l, s);
            }
        }
        if (cudaGetLastError() != cudaSuccess) st = TSQR_ERR_CUDA;
    }
    delete ft;
    delete at;
    return st;
}

}  // namespace tsqr
