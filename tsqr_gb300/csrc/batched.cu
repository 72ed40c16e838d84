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
#include <mutex>
#include <vector>

#include "internal.h"
#include "tsqr_kernels.cuh"

namespace tsqr {

namespace {

constexpr int kTable = 448;  // descriptors per launch (fits the 32 KB parameter space)
constexpr int kBatchedCands = 2;    // tile configurations per width class
constexpr int kBatchedBuckets = 3;  // problem-height buckets of the tuning table

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
    pdl_begin();
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
    pdl_begin();
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
    pdl_begin();
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
    static PerDeviceOnce attr;
    attr.run([] {
        cudaFuncSetAttribute(batched_apply<NMAX, ANT, ARPT, AMINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmem);
    });
    launch_pdl(batched_apply<NMAX, ANT, ARPT, AMINB>, dim3(grid), dim3(ANT), kSmem, s, t);
}

// one thread per row slice (factor_tile)
template <int NMAX, int NT, int RPT, int MINB, int AMINB, int ANT = NT>
struct Cls {
    static void factor(const FactorTable& t, int grid, cudaStream_t s) {
        launch_pdl(batched_factor<NMAX, NT, RPT, MINB>, dim3(grid), dim3(NT), 0, s, t);
    }
    static ClassCfg cfg() { return {NMAX, NT * RPT, MINB, AMINB, &factor, &class_apply<NMAX, NT * RPT, ANT, AMINB>}; }
};

// column-split tiles (factor_split_tile)
template <int NMAX, int CW, int RPT, int MINB, int AMINB, int ANT>
struct SplitCls {
    static void factor(const FactorTable& t, int grid, cudaStream_t s) {
        launch_pdl(batched_factor_split<NMAX, CW, RPT, MINB>, dim3(grid), dim3(32 * (NMAX / CW)), 0, s, t);
    }
    static ClassCfg cfg() { return {NMAX, 32 * RPT, MINB, AMINB, &factor, &class_apply<NMAX, 32 * RPT, ANT, AMINB>}; }
};

// Candidate tile configurations per width class (n <= 8, 16, 32, 64).
// Candidate 0 is the single-problem path's configuration; candidate 1 halves
// the tile height (more tiles, hence more parallelism, for short problems,
// at the cost of a taller stacked-R level).
int class_index(int n) { return n <= 8 ? 0 : (n <= 16 ? 1 : (n <= 32 ? 2 : 3)); }

const ClassCfg& candidate(int ci, int cand) {
    static const ClassCfg c[4][kBatchedCands] = {
        {Cls<8, 256, 4, 3, 3>::cfg(), Cls<8, 256, 2, 3, 3>::cfg()},
        {SplitCls<16, 4, 16, 4, 3, 256>::cfg(), SplitCls<16, 4, 8, 4, 3, 256>::cfg()},
        {SplitCls<32, 4, 16, 2, 2, 256>::cfg(), SplitCls<32, 4, 8, 2, 2, 256>::cfg()},
        {SplitCls<64, 8, 16, 1, 1, 256>::cfg(), SplitCls<64, 8, 8, 1, 1, 256>::cfg()},
    };
    return c[ci][cand];
}

// Height bucket of a problem: m < 8192, m < 65536, m >= 65536.
int bucket_of(int64_t m) { return m < 8192 ? 0 : (m < 65536 ? 1 : 2); }

// The autotuner's table: candidate per (class, bucket), candidate 0 until a
// tuning call or tsqr_batched_set_choice changes it.  Process-wide.
std::mutex g_table_mu;
int g_table[4][kBatchedBuckets] = {};

int choice_of(int ci, int bk) {
    std::lock_guard<std::mutex> g(g_table_mu);
    return g_table[ci][bk];
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
    const int sms = device_sm_count();
    const int per_sm = apply ? c.apply_per_sm : c.factor_per_sm;
    return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sms * per_sm));
}

}  // namespace

// Sized for the largest candidate of each problem, so the answer holds
// whatever the tuning table says when the call runs.
size_t batched_workspace(int count, const int64_t* m, const int64_t* n) {
    size_t total = 0;
    for (int i = 0; i < count; ++i) {
        if (m[i] < 1 || n[i] < 1 || n[i] > 64 || m[i] < n[i]) return 0;
        size_t most = 0;
        for (int c = 0; c < kBatchedCands; ++c)
            most = std::max(most, tree_of(m[i], n[i], nullptr, m[i], candidate(class_index((int)n[i]), c).rows,
                                          nullptr, nullptr));
        total += most;
    }
    return total < 256 ? 256 : total;
}

tsqr_status batched_run(int count, float* const* A, const int64_t* m, const int64_t* n, const int64_t* lda,
                        float* const* R, const int64_t* ldr, void* work, size_t work_bytes, cudaStream_t s) {
    if (count == 0) return TSQR_OK;
    const size_t need = batched_workspace(count, m, n);
    if (need == 0) return TSQR_ERR_INVALID_ARG;
    if (work == nullptr || work_bytes < need) return TSQR_ERR_WORKSPACE;
    // One snapshot of the tuning table for the whole call.
    int table[4][kBatchedBuckets];
    {
        std::lock_guard<std::mutex> g(g_table_mu);
        std::copy(&g_table[0][0], &g_table[0][0] + 4 * kBatchedBuckets, &table[0][0]);
    }
    std::vector<int> cand_of(count);
    for (int i = 0; i < count; ++i) cand_of[i] = table[class_index((int)n[i])][bucket_of(m[i])];
    // Trees of every problem.
    std::vector<std::vector<Lvl>> trees(count);
    char* base = reinterpret_cast<char*>(work);
    size_t off = 0;
    for (int i = 0; i < count; ++i)
        off += tree_of(m[i], n[i], A[i], lda[i], candidate(class_index((int)n[i]), cand_of[i]).rows, base + off,
                       &trees[i]);

    FactorTable* ft = new FactorTable;
    ApplyTable* at = new ApplyTable;
    tsqr_status st = TSQR_OK;
    // one group per (width class, candidate configuration)
    for (int g = 0; g < 4 * kBatchedCands && st == TSQR_OK; ++g) {
        const int ci = g / kBatchedCands, cand = g % kBatchedCands;
        std::vector<int> members;
        for (int i = 0; i < count; ++i)
            if (class_index((int)n[i]) == ci && cand_of[i] == cand) members.push_back(i);
        if (members.empty()) continue;
        const ClassCfg& C = candidate(ci, cand);
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

namespace {

__global__ void fill_uniform_kernel(float* a, int64_t count, uint32_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t x = (uint32_t)i * 2654435761u ^ (uint32_t)(i >> 32) ^ seed;
        x ^= x >> 15;
        x *= 2246822519u;
        x ^= x >> 13;
        a[i] = (float)(x >> 8) * (2.0f / 16777216.0f) - 1.0f;
    }
}

}  // namespace

// Times every candidate configuration of each (width class, height bucket)
// present in the given shapes on synthetic matrices of those shapes, and
// keeps the fastest in the table.  Allocates its own scratch.
tsqr_status batched_tune(int count, const int64_t* m, const int64_t* n, int reps, cudaStream_t s) {
    if (count < 1 || !m || !n || reps < 1) return TSQR_ERR_INVALID_ARG;
    for (int i = 0; i < count; ++i)
        if (m[i] < 1 || n[i] < 1 || n[i] > 64 || m[i] < n[i] || m[i] > INT32_MAX) return TSQR_ERR_INVALID_ARG;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return TSQR_ERR_CUDA;
    tsqr_status st = TSQR_OK;
    for (int ci = 0; ci < 4 && st == TSQR_OK; ++ci)
        for (int bk = 0; bk < kBatchedBuckets && st == TSQR_OK; ++bk) {
            std::vector<int64_t> mm, nn, ld, ldr;
            for (int i = 0; i < count; ++i)
                if (class_index((int)n[i]) == ci && bucket_of(m[i]) == bk) {
                    mm.push_back(m[i]);
                    nn.push_back(n[i]);
                }
            if (mm.empty()) continue;
            const int k = (int)mm.size();
            int64_t elems = 0, relems = 0;
            for (int i = 0; i < k; ++i) elems += mm[i] * nn[i], relems += nn[i] * nn[i];
            const size_t wb = batched_workspace(k, mm.data(), nn.data());
            float *dA = nullptr, *dR = nullptr;
            void* dW = nullptr;
            if (cudaMalloc(&dA, sizeof(float) * elems) != cudaSuccess ||
                cudaMalloc(&dR, sizeof(float) * relems) != cudaSuccess || cudaMalloc(&dW, wb) != cudaSuccess) {
                st = TSQR_ERR_CUDA;
            } else {
                std::vector<float*> pa(k), pr(k);
                int64_t oa = 0, orr = 0;
                for (int i = 0; i < k; ++i) {
                    pa[i] = dA + oa;
                    pr[i] = dR + orr;
                    oa += mm[i] * nn[i];
                    orr += nn[i] * nn[i];
                    ld.push_back(mm[i]);
                    ldr.push_back(nn[i]);
                }
                int best = 0;
                float best_ms = 0.f;
                for (int cand = 0; cand < kBatchedCands && st == TSQR_OK; ++cand) {
                    {
                        std::lock_guard<std::mutex> g(g_table_mu);
                        g_table[ci][bk] = cand;
                    }
                    float total = 0.f;
                    for (int r = 0; r <= reps && st == TSQR_OK; ++r) {  // r = 0 is a warm-up
                        fill_uniform_kernel<<<1024, 256, 0, s>>>(dA, elems, 977u * (uint32_t)(r + 1));
                        cudaEventRecord(e0, s);
                        st = batched_run(k, pa.data(), mm.data(), nn.data(), ld.data(), pr.data(), ldr.data(), dW, wb,
                                         s);
                        cudaEventRecord(e1, s);
                        if (st == TSQR_OK && cudaEventSynchronize(e1) != cudaSuccess) st = TSQR_ERR_CUDA;
                        float ms = 0.f;
                        if (st == TSQR_OK && r > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) total += ms;
                    }
                    if (st == TSQR_OK && (cand == 0 || total < best_ms)) best = cand, best_ms = total;
                }
                std::lock_guard<std::mutex> g(g_table_mu);
                g_table[ci][bk] = best;
            }
            cudaFree(dA);
            cudaFree(dR);
            cudaFree(dW);
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
}

int batched_choice(int ci, int bk) {
    if (ci < 0 || ci >= 4 || bk < 0 || bk >= kBatchedBuckets) return -1;
    return choice_of(ci, bk);
}

int batched_candidate_rows(int ci, int cand) {
    if (ci < 0 || ci >= 4 || cand < 0 || cand >= kBatchedCands) return -1;
    return candidate(ci, cand).rows;
}

tsqr_status batched_set_choice(int ci, int bk, int cand) {
    if (ci < 0 || ci >= 4 || bk < 0 || bk >= kBatchedBuckets || cand < 0 || cand >= kBatchedCands)
        return TSQR_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(g_table_mu);
    g_table[ci][bk] = cand;
    return TSQR_OK;
}

}  // namespace tsqr
