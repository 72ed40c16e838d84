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

// cuTensorMapEncodeTiled, looked up once through the runtime (no link
// against the driver library).  Null if the driver does not offer it.
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        (void)cudaGetLastError();
        return reinterpret_cast<EncodeTiledFn>(f);
    }();
    return fn;
}

}  // namespace

bool tensor_map_f32(CUtensorMap* map, const float* base, int64_t ld, int64_t rows, int64_t cols, int box_rows,
                    int box_cols, bool swizzle128) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc || (reinterpret_cast<uintptr_t>(base) % 16) != 0 || ld % 4 != 0 || rows < 1 || cols < 1) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
    const cuuint32_t estr[2] = {1u, 1u};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace {

// Tensor map of an FP32 level matrix (h rows x n columns) for boxes of 256
// rows x nbox columns.
bool level_tensor_map(CUtensorMap* map, const float* M, int64_t ld, int64_t h, int n, int nbox) {
    return tensor_map_f32(map, M, ld, h, n, 256, nbox, false);
}

template <typename T, int NMAX, int NT, int RPT, int MINB, int AMINB, int ANT = NT, bool NORM64 = false>
struct TileCfg {
    static_assert((NT * RPT) % ANT == 0, "apply block must divide the tile");
    static constexpr int ARPT = NT * RPT / ANT;
    static constexpr int kRows = NT * RPT;
    static void factor(const FactorParams<T>& p, int grid, cudaStream_t s) {
        launch_pdl(factor_tiles<T, NMAX, NT, RPT, MINB, NORM64>, dim3(grid), dim3(NT), 0, s, p);
    }
    static void apply(const ApplyParams<T>& p, int grid, cudaStream_t s) {
        constexpr size_t smem = apply_smem_bytes<T, NMAX, ANT * ARPT>();
        static PerDeviceOnce attr;
        attr.run([] {
            cudaFuncSetAttribute(apply_tiles<T, NMAX, ANT, ARPT, AMINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        });
        launch_pdl(apply_tiles<T, NMAX, ANT, ARPT, AMINB>, dim3(grid), dim3(ANT), smem, s, p);
    }
};

// Factor on column-split tiles (factor_split_tiles: NMAX/CW warps per
// 32*RPT-row tile), with the same apply kernel as TileCfg.
template <typename T, int NMAX, int CW, int RPT, int MINB, int ANT, int AMINB, bool N64 = false>
struct SplitCfg {
    static constexpr int kRows = 32 * RPT;
    static constexpr int ARPT = kRows / ANT;
    static_assert(kRows % ANT == 0, "apply block must divide the tile");
    static void factor(const FactorParams<T>& p, int grid, cudaStream_t s) {
        // A single-tile level (the root) of h rows takes the same kernel with
        // just enough rows per lane (32 * rpt >= h): every step issues the
        // FMAs of all RPT rows of a lane, so a 64-row root on the 512-row
        // kernel would spend 7/8 of them on zero rows.
        constexpr int W32 = 32 * (NMAX / CW);
        if constexpr (RPT > 2 && NMAX <= 64)
            if (p.ntiles == 1 && p.h <= 64)
                return (void)launch_pdl(factor_split_tiles<T, NMAX, CW, 2, 1, N64>, dim3(1), dim3(W32), 0, s, p);
        if constexpr (RPT > 4)
            if (p.ntiles == 1 && p.h <= 128)
                return (void)launch_pdl(factor_split_tiles<T, NMAX, CW, 4, 1, N64>, dim3(1), dim3(W32), 0, s, p);
        if constexpr (RPT > 8)
            if (p.ntiles == 1 && p.h <= 256)
                return (void)launch_pdl(factor_split_tiles<T, NMAX, CW, 8, 1, N64>, dim3(1), dim3(W32), 0, s, p);
        if constexpr (std::is_same<T, float>::value && RPT == 16 && NMAX <= 32 && !N64) {
            // levels with several tiles per resident CTA: tiles staged by TMA
            // into shared memory, the next one copied while the current one
            // is factored (persistent CTAs).  Measured at 4,194,304 x 32:
            // level 0 0.670 ms against 0.667 ms with register loads, so the
            // staging costs nothing there; levels of one wave or less were
            // 2 us slower with it and keep the plain loads.
            const int64_t resident = (int64_t)device_sm_count() * MINB;
            CUtensorMap map;
            if (p.ntiles >= 2 * resident && p.ntiles * kRows <= INT32_MAX &&
                level_tensor_map(&map, p.M, p.ld, p.h, p.n, NMAX)) {
                constexpr size_t smem = tma_stage_bytes<T, NMAX, CW, RPT>();
                static PerDeviceOnce attr;
                attr.run([] {
                    cudaFuncSetAttribute(factor_split_tiles_tma<T, NMAX, CW, RPT, MINB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                });
                const int g = (int)std::min<int64_t>(p.ntiles, resident);
                return (void)launch_pdl(factor_split_tiles_tma<T, NMAX, CW, RPT, MINB>, dim3(g), dim3(W32), smem, s,
                                        p, map);
            }
        }
        launch_pdl(factor_split_tiles<T, NMAX, CW, RPT, MINB, N64>, dim3(grid), dim3(W32), 0, s, p);
    }
    static void apply(const ApplyParams<T>& p, int grid, cudaStream_t s) {
        TileCfg<T, NMAX, ANT, ARPT, 1, AMINB>::apply(p, grid, s);
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
    // Level-0 factor times at 4,194,304 rows, column-split (factor_split_tiles)
    // against the earlier one-thread-per-row-slice kernel (factor_tiles):
    // n = 16: 0.20 vs 0.49 ms; n = 32: 0.72 vs 0.98 ms; n = 64: 3.2 vs 5.7 ms.
    // n = 64 keeps 512-row tiles (whole TSQR 6.9 ms, vs 9.9 ms with 256-row
    // tiles, whose stacked-R level is twice as tall).
    if (n <= 8) return make_set<TileCfg<float, 8, 256, 4, 3, 3>, float>();
    if (n <= 16) return make_set<SplitCfg<float, 16, 4, 16, 4, 256, 3>, float>();
    if (n <= 32) return make_set<SplitCfg<float, 32, 4, 16, 2, 256, 2>, float>();
    if (n <= 64) return make_set<SplitCfg<float, 64, 8, 16, 1, 256, 1>, float>();
    return KernelSet<float>();
}
KernelSet<double> pick(double*, int n) {
    // n = 32 at 2,097,152 rows: 7.5 ms (column-split) vs 19.0 ms
    if (n <= 8) return make_set<TileCfg<double, 8, 256, 2, 2, 3>, double>();
    if (n <= 16) return make_set<TileCfg<double, 16, 256, 2, 1, 2>, double>();
    if (n <= 32) return make_set<SplitCfg<double, 32, 4, 8, 3, 256, 2>, double>();
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

// Workspace of the plain tree: a status word (256 bytes; non-zero after a
// factor kernel's bounded wait gave up, read by tsqr_workspace_check), then
// the level matrices.
template <typename T>
size_t tsqr_plain_workspace(int64_t m, int64_t n) {
    KernelSet<T> ks = pick((T*)nullptr, (int)n);
    if (!ks.factor) return 0;
    return kAlign + plan_levels<T>(m, n, nullptr, m, ks.rows, nullptr, nullptr);
}

template <typename T>
tsqr_status tsqr_plain(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                       cudaStream_t s, int phases) {
    const PdlOff no_pdl(n > 32);
    KernelSet<T> ks = pick((T*)nullptr, (int)n);
    if (!ks.factor) return TSQR_ERR_UNSUPPORTED;
    std::vector<Level<T>> lv;
    char* wb = reinterpret_cast<char*>(work);
    size_t need = plan_levels<T>(m, n, A, lda, ks.rows, wb ? wb + kAlign : nullptr, &lv);
    if (need > 0 && (work == nullptr || work_bytes < kAlign + need)) return TSQR_ERR_WORKSPACE;
    // a single-tile problem may run without a workspace, and then without a
    // status word
    int* err = (work != nullptr && work_bytes >= kAlign) ? reinterpret_cast<int*>(work) : nullptr;
    if (err && (phases & kPhaseUp) && cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return TSQR_ERR_CUDA;
    const int L = (int)lv.size();
    // up-sweep
    for (int l = 0; l < L && (phases & kPhaseUp); ++l) {
        FactorParams<T> fp;
        fp.M = lv[l].M;
        fp.ld = lv[l].ld;
        fp.h = lv[l].h;
        fp.n = (int)n;
        fp.ntiles = lv[l].ntiles;
        fp.err = err;
        fp.tries = wait_tries().load(std::memory_order_relaxed);
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
    for (int l = L - 1; l >= 0 && (phases & kPhaseDown); --l) {
        ApplyParams<T> ap;
        ap.M = lv[l].M;
        ap.ld = lv[l].ld;
        ap.h = lv[l].h;
        ap.n = (int)n;
        ap.ntiles = lv[l].ntiles;
        ap.P = (l == L - 1) ? nullptr : lv[l + 1].M;
        ap.ldp = (l == L - 1) ? 0 : lv[l + 1].ld;
        constexpr int ve = 16 / sizeof(T);
        ap.vec = (lv[l].ld % ve == 0 && (reinterpret_cast<uintptr_t>(lv[l].M) % 16) == 0) ? 1 : 0;
        ks.apply(ap, (int)std::min<int64_t>(lv[l].ntiles, 1 << 30), s);
        log_launch(kTagApply + l, s);
    }
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Precision form (FP32 entry points): the tile factorisation stays FP32 on
// CUDA cores; every Q assembly of the down-sweep runs on tcgen05 in TF32x3
// (tc_apply.cu).  An FP64 root combine (the last level converted to double
// and factored by the FP64 tree) is built in but switched off (kRoot64).
// Workspace: [status word (256 B) | level matrices | FP64 root copy | FP64
// root-tree workspace].
// ---------------------------------------------------------------------------
namespace {

template <typename A, typename B>
__global__ void convert_matrix(int64_t h, int n, const A* __restrict__ src, int64_t lds, B* __restrict__ dst,
                               int64_t ldd) {
    const int64_t total = h * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e % h, c = e / h;
        dst[r + c * ldd] = (B)src[r + c * lds];
    }
}

template <typename A, typename B>
void convert(int64_t h, int n, const A* src, int64_t lds, B* dst, int64_t ldd, cudaStream_t s) {
    const int64_t total = h * n;
    const int blocks = (int)std::min<int64_t>(ceil_div(total, 256), 1024);
    convert_matrix<A, B><<<blocks, 256, 0, s>>>(h, n, src, lds, dst, ldd);
}

struct PrecCfg {
    int nmax = 0, rows = 0;
    KernelSet<float> ks;
};

// The tile factorisation is the plain FP32 kernel; with norm64
// (tsqr_opts.fp64_scalars) its variant whose per-column norm, beta and tau
// are computed in FP64.
PrecCfg pick_precision(int n, bool norm64 = false) {
    PrecCfg c;
    if (n <= 16) {
        c.nmax = 16;
        c.ks = norm64 ? make_set<SplitCfg<float, 16, 4, 16, 4, 256, 3, true>, float>()
                      : make_set<SplitCfg<float, 16, 4, 16, 4, 256, 3>, float>();
    } else if (n <= 32) {
        c.nmax = 32;
        c.ks = norm64 ? make_set<SplitCfg<float, 32, 4, 16, 2, 256, 2, true>, float>()
                      : make_set<SplitCfg<float, 32, 4, 16, 2, 256, 2>, float>();
    } else if (n <= 64) {
        c.nmax = 64;
        c.ks = norm64 ? make_set<SplitCfg<float, 64, 8, 16, 1, 256, 1, true>, float>()
                      : make_set<SplitCfg<float, 64, 8, 16, 1, 256, 1>, float>();
    }
    c.rows = c.ks.rows;
    return c;
}

struct PrecLayout {
    size_t status = 0, levels = 0, root = 0, rootws = 0, total = 0;
};

// Root combine in FP64 (tsqr_opts.fp64_root, n <= 32): the root level
// converted to double, factored by the FP64 tree, converted back.
PrecLayout prec_layout(int64_t m, int64_t n, const PrecCfg& c, bool root64_opt = false) {
    PrecLayout L;
    L.status = 0;
    L.levels = kAlign;
    std::vector<Level<float>> lv;
    const size_t lev = plan_levels<float>(m, n, nullptr, m, c.rows, nullptr, &lv);
    L.root = L.levels + lev;
    const int64_t hroot = lv.back().h;
    const bool root64 = root64_opt && n <= 32;
    const size_t rootbytes = root64 ? (size_t)round_up(hroot * n * 8 + n * n * 8, (int64_t)kAlign) : 0;
    L.rootws = L.root + rootbytes;
    L.total = L.rootws + (root64 ? round_up((int64_t)tsqr_plain_workspace<double>(hroot, n), (int64_t)kAlign) : 0);
    return L;
}

}  // namespace

bool tc_apply_level(const ApplyParams<float>& p, int nmax, int rows, int* err, cudaStream_t s);

size_t tsqr_precision_workspace(int64_t m, int64_t n, PrecFlags f) {
    PrecCfg c = pick_precision((int)n, f.norm64);
    if (!c.ks.factor) return 0;
    return prec_layout(m, n, c, f.root64).total;
}

tsqr_status tsqr_precision(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                           size_t work_bytes, cudaStream_t s, PrecFlags f) {
    const PdlOff no_pdl(n > 32);
    PrecCfg c = pick_precision((int)n, f.norm64);
    if (!c.ks.factor) return TSQR_ERR_UNSUPPORTED;
    if (f.root64 && n > 32) return TSQR_ERR_UNSUPPORTED;
    const PrecLayout PL = prec_layout(m, n, c, f.root64);
    if (work == nullptr || work_bytes < PL.total) return TSQR_ERR_WORKSPACE;
    char* base = reinterpret_cast<char*>(work);
    int* err = reinterpret_cast<int*>(base + PL.status);
    std::vector<Level<float>> lv;
    plan_levels<float>(m, n, A, lda, c.rows, base + PL.levels, &lv);
    const int L = (int)lv.size();
    if (f.clear_status && cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return TSQR_ERR_CUDA;
    const bool root64 = f.root64;
    const int top = root64 ? L - 1 : L;  // levels factored in FP32 below the root
    for (int l = 0; l < top; ++l) {
        FactorParams<float> fp;
        fp.M = lv[l].M;
        fp.ld = lv[l].ld;
        fp.h = lv[l].h;
        fp.n = (int)n;
        fp.ntiles = lv[l].ntiles;
        fp.err = err;
        fp.tries = wait_tries().load(std::memory_order_relaxed);
        fp.Rout = (l == L - 1) ? R : lv[l + 1].M;
        fp.ldr = (l == L - 1) ? ldr : lv[l + 1].ld;
        c.ks.factor(fp, (int)std::min<int64_t>(lv[l].ntiles, 1 << 30), s);
        log_launch(kTagFactor + l, s);
    }
    if (root64) {
        // FP64 root combine: the last level (at most one tile of stacked R
        // factors, or A itself when m fits one tile) factored in double.
        const Level<float>& rt = lv[L - 1];
        double* Qd = reinterpret_cast<double*>(base + PL.root);
        double* Rd = Qd + rt.h * n;
        convert<float, double>(rt.h, (int)n, rt.M, rt.ld, Qd, rt.h, s);
        log_launch(kTagTc + 900, s);
        tsqr_status st = tsqr_plain<double>(rt.h, n, Qd, rt.h, Rd, n, base + PL.rootws, PL.total - PL.rootws, s);
        if (st != TSQR_OK) return st;
        convert<double, float>(rt.h, (int)n, Qd, rt.h, rt.M, rt.ld, s);
        convert<double, float>(n, (int)n, Rd, n, R, ldr, s);
        log_launch(kTagTc + 901, s);
    }
    for (int l = (root64 ? L - 2 : L - 1); l >= 0; --l) {
        ApplyParams<float> ap;
        ap.M = lv[l].M;
        ap.ld = lv[l].ld;
        ap.h = lv[l].h;
        ap.n = (int)n;
        ap.ntiles = lv[l].ntiles;
        ap.P = (l == L - 1) ? nullptr : lv[l + 1].M;
        ap.ldp = (l == L - 1) ? 0 : lv[l + 1].ld;
        ap.vec = 0;
        if (!tc_apply_level(ap, c.nmax, c.rows, err, s)) return TSQR_ERR_UNSUPPORTED;
        log_launch(kTagTc + l, s);
    }
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

template size_t tsqr_plain_workspace<float>(int64_t, int64_t);
template size_t tsqr_plain_workspace<double>(int64_t, int64_t);
template <typename T>
tsqr_status tsqr_plain_tree(int64_t m, int64_t n, const T* A, int64_t lda, const void* work, size_t work_bytes,
                            std::vector<TreeLevel<T>>* out) {
    KernelSet<T> ks = pick((T*)nullptr, (int)n);
    if (!ks.factor) return TSQR_ERR_UNSUPPORTED;
    std::vector<Level<T>> lv;
    char* wb = const_cast<char*>(reinterpret_cast<const char*>(work));
    size_t need = plan_levels<T>(m, n, const_cast<T*>(A), lda, ks.rows, wb ? wb + kAlign : nullptr, &lv);
    if (need > 0 && (work == nullptr || work_bytes < kAlign + need)) return TSQR_ERR_WORKSPACE;
    out->clear();
    for (const Level<T>& v : lv) out->push_back({v.M, v.ld, v.h, v.ntiles, ks.rows});
    return TSQR_OK;
}
template tsqr_status tsqr_plain_tree<float>(int64_t, int64_t, const float*, int64_t, const void*, size_t,
                                            std::vector<TreeLevel<float>>*);
template tsqr_status tsqr_plain_tree<double>(int64_t, int64_t, const double*, int64_t, const void*, size_t,
                                             std::vector<TreeLevel<double>>*);
template tsqr_status tsqr_plain<float>(int64_t, int64_t, float*, int64_t, float*, int64_t, void*, size_t,
                                       cudaStream_t, int);
template tsqr_status tsqr_plain<double>(int64_t, int64_t, double*, int64_t, double*, int64_t, void*, size_t,
                                        cudaStream_t, int);

// ---------------------------------------------------------------------------
// TSQR of a matrix in host memory (tsqr_s_host / tsqr_d_host).  The device
// holds a copy of A (ld rounded up to 32 rows), the n x n R and the tree.
// Level 0 is cut into chunks of whole tiles.  A library copy stream moves
// chunk c to the device while the caller's stream factors chunk c-1; after
// the upper levels, the caller's stream assembles Q chunk by chunk while the
// copy stream returns the finished chunks, so both host transfers overlap
// the level-0 kernels instead of adding to them.  The copy stream and its
// events belong to the calling host thread (one set per device), so calls
// from different threads share nothing; a problem of one chunk copies on
// the caller's stream alone.
// ---------------------------------------------------------------------------
namespace {

constexpr int kHostChunks = 8;
constexpr int64_t kHostChunkBytes = 16 << 20;

// Copy stream and events of one host thread on one device.
struct HostPipe {
    int dev = -1;
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[2 * kHostChunks + 2] = {};
};

HostPipe* host_pipe() {
    thread_local HostPipe pipes[8];
    thread_local int used = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    for (int i = 0; i < used; ++i)
        if (pipes[i].dev == dev) return &pipes[i];
    if (used == 8) return nullptr;
    HostPipe& p = pipes[used];
    if (cudaStreamCreateWithFlags(&p.cs, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    for (auto& e : p.ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    p.dev = dev;
    ++used;
    return &p;
}

template <typename T>
struct HostLayout {
    int64_t ldd = 0;
    size_t a = 0, r = 0, tree = 0, total = 0;
};

// The tree comes first, so the precision form's status word sits at the
// start of the workspace as for the device entry points.
template <typename T>
HostLayout<T> host_layout(int64_t m, int64_t n, bool prec) {
    HostLayout<T> L;
    L.ldd = round_up(m, 32);
    size_t tw = 0;
    if constexpr (sizeof(T) == 4) {
        if (prec) {
            PrecCfg c = pick_precision((int)n);
            tw = c.ks.factor ? prec_layout(m, n, c).total : 0;
        }
    }
    if (!prec) tw = tsqr_plain_workspace<T>(m, n);
    L.tree = 0;
    L.a = (size_t)round_up((int64_t)tw, (int64_t)kAlign);
    L.r = L.a + (size_t)round_up(L.ldd * n * (int64_t)sizeof(T), (int64_t)kAlign);
    const size_t end = L.r + (size_t)round_up(n * n * (int64_t)sizeof(T), (int64_t)kAlign);
    L.total = tw ? end : 0;
    return L;
}

}  // namespace

template <typename T>
size_t tsqr_host_workspace(int64_t m, int64_t n, bool prec) {
    return host_layout<T>(m, n, prec).total;
}

template <typename T>
tsqr_status tsqr_host(int64_t m, int64_t n, const T* hA, int64_t lda, T* hQ, int64_t ldq, T* hR, int64_t ldr,
                      void* work, size_t work_bytes, bool prec, cudaStream_t s) {
    const PdlOff no_pdl;  // the kernels below wait on the copy stream's events
    const HostLayout<T> HL = host_layout<T>(m, n, prec);
    if (HL.total == 0) return TSQR_ERR_UNSUPPORTED;
    if (work == nullptr || work_bytes < HL.total) return TSQR_ERR_WORKSPACE;
    char* base = reinterpret_cast<char*>(work);
    T* dA = reinterpret_cast<T*>(base + HL.a);
    T* dR = reinterpret_cast<T*>(base + HL.r);
    char* tw = base + HL.tree;

    // the tree of the chosen form
    KernelSet<T> ks;
    int nmax = 0;
    bool tc = false;
    int* err = nullptr;
    char* lvbase = tw;
    if constexpr (sizeof(T) == 4) {
        if (prec) {
            PrecCfg c = pick_precision((int)n);
            const PrecLayout PL = prec_layout(m, n, c);
            ks = c.ks;
            nmax = c.nmax;
            tc = true;
            err = reinterpret_cast<int*>(tw + PL.status);
            lvbase = tw + PL.levels;
        }
    }
    if (!prec) {
        ks = pick((T*)nullptr, (int)n);
        err = reinterpret_cast<int*>(tw);  // the plain tree's status word
        lvbase = tw + kAlign;
    }
    if (!ks.factor) return TSQR_ERR_UNSUPPORTED;
    std::vector<Level<T>> lv;
    plan_levels<T>(m, n, dA, HL.ldd, ks.rows, lvbase, &lv);
    const int L = (int)lv.size();
    const int64_t rows = ks.rows;

    auto factor = [&](int l, int64_t t0, int64_t cnt) {
        FactorParams<T> fp;
        fp.M = lv[l].M + t0 * rows;
        fp.ld = lv[l].ld;
        fp.h = std::min<int64_t>(cnt * rows, lv[l].h - t0 * rows);
        fp.n = (int)n;
        fp.ntiles = cnt;
        fp.err = err;
        fp.tries = wait_tries().load(std::memory_order_relaxed);
        fp.Rout = (l == L - 1) ? dR : lv[l + 1].M + t0 * n;
        fp.ldr = (l == L - 1) ? n : lv[l + 1].ld;
        ks.factor(fp, (int)std::min<int64_t>(cnt, 1 << 30), s);
        log_launch(kTagFactor + l, s);
    };
    auto apply = [&](int l, int64_t t0, int64_t cnt) -> bool {
        ApplyParams<T> ap;
        ap.M = lv[l].M + t0 * rows;
        ap.ld = lv[l].ld;
        ap.h = std::min<int64_t>(cnt * rows, lv[l].h - t0 * rows);
        ap.n = (int)n;
        ap.ntiles = cnt;
        ap.P = (l == L - 1) ? nullptr : lv[l + 1].M + t0 * n;
        ap.ldp = (l == L - 1) ? 0 : lv[l + 1].ld;
        if constexpr (sizeof(T) == 4) {
            if (tc) {
                ap.vec = 0;
                if (!tc_apply_level(ap, nmax, (int)rows, err, s)) return false;
                log_launch(kTagTc + l, s);
                return true;
            }
        }
        constexpr int ve = 16 / sizeof(T);
        ap.vec = (ap.ld % ve == 0 && (reinterpret_cast<uintptr_t>(ap.M) % 16) == 0) ? 1 : 0;
        ks.apply(ap, (int)std::min<int64_t>(cnt, 1 << 30), s);
        log_launch(kTagApply + l, s);
        return true;
    };

    const int64_t nt0 = lv[0].ntiles;
    // chunks of at least kHostChunkBytes: smaller copies gain less from the
    // overlap than the extra launches and stream operations cost
    const int64_t by_size = std::max<int64_t>(1, (m * n * (int64_t)sizeof(T)) / kHostChunkBytes);
    const int nc = (int)std::min<int64_t>(std::min<int64_t>(kHostChunks, nt0), by_size);
    const int64_t per = ceil_div(nt0, nc);
    const size_t es = sizeof(T);
    tsqr_status st = TSQR_OK;
    // One chunk leaves nothing to overlap: copies on the caller's stream.
    // Otherwise the copy stream and events of this host thread (made once per
    // thread and device, reused by its later calls: a host thread issues its
    // calls one after another, and a wait captures an event's state when it
    // is enqueued, so re-recording an event cannot disturb an earlier call).
    cudaStream_t cs = s;
    cudaEvent_t* ev = nullptr;
    if (nc > 1) {
        HostPipe* hp = host_pipe();
        if (!hp) return TSQR_ERR_CUDA;
        cs = hp->cs;
        ev = hp->ev;
    }
    if (nc == 1) {
        const int64_t hr = m;
        if (cudaMemcpy2DAsync(dA, HL.ldd * es, hA, lda * es, hr * es, n, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return TSQR_ERR_CUDA;
        if (err) cudaMemsetAsync(err, 0, sizeof(int), s);
        for (int l = 0; l < L; ++l) factor(l, 0, lv[l].ntiles);
        for (int l = L - 1; l >= 0; --l)
            if (!apply(l, 0, lv[l].ntiles)) return TSQR_ERR_UNSUPPORTED;
        if (cudaMemcpy2DAsync(hR, ldr * es, dR, n * es, n * es, n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpy2DAsync(hQ, ldq * es, dA, HL.ldd * es, hr * es, n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return TSQR_ERR_CUDA;
        return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
    }
    {
        // the copy stream starts after the caller's earlier work
        cudaEventRecord(ev[2 * kHostChunks], s);
        cudaStreamWaitEvent(cs, ev[2 * kHostChunks], 0);
        if (err) cudaMemsetAsync(err, 0, sizeof(int), s);
        // up: chunk c copied in while chunk c-1 is factored
        for (int c = 0; c < nc; ++c) {
            const int64_t t0 = c * per, cnt = std::min<int64_t>(per, nt0 - t0);
            if (cnt <= 0) break;
            const int64_t r0 = t0 * rows, hr = std::min<int64_t>(cnt * rows, m - r0);
            if (cudaMemcpy2DAsync(dA + r0, HL.ldd * es, hA + r0, lda * es, hr * es, n, cudaMemcpyHostToDevice, cs) !=
                cudaSuccess)
                st = TSQR_ERR_CUDA;
            cudaEventRecord(ev[c], cs);
            cudaStreamWaitEvent(s, ev[c], 0);
            factor(0, t0, cnt);
        }
        for (int l = 1; l < L; ++l) factor(l, 0, lv[l].ntiles);
        for (int l = L - 1; l >= 1 && st == TSQR_OK; --l)
            if (!apply(l, 0, lv[l].ntiles)) st = TSQR_ERR_UNSUPPORTED;
        if (cudaMemcpy2DAsync(hR, ldr * es, dR, n * es, n * es, n, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            st = TSQR_ERR_CUDA;
        // down: chunk c of Q returned while chunk c+1 is assembled
        for (int c = 0; c < nc && st == TSQR_OK; ++c) {
            const int64_t t0 = c * per, cnt = std::min<int64_t>(per, nt0 - t0);
            if (cnt <= 0) break;
            const int64_t r0 = t0 * rows, hr = std::min<int64_t>(cnt * rows, m - r0);
            if (!apply(0, t0, cnt)) {
                st = TSQR_ERR_UNSUPPORTED;
                break;
            }
            cudaEventRecord(ev[kHostChunks + c], s);
            cudaStreamWaitEvent(cs, ev[kHostChunks + c], 0);
            if (cudaMemcpy2DAsync(hQ + r0, ldq * es, dA + r0, HL.ldd * es, hr * es, n, cudaMemcpyDeviceToHost, cs) !=
                cudaSuccess)
                st = TSQR_ERR_CUDA;
        }
        // the caller's stream completes after the last copy
        cudaEventRecord(ev[2 * kHostChunks + 1], cs);
        cudaStreamWaitEvent(s, ev[2 * kHostChunks + 1], 0);
    }
    if (st != TSQR_OK) return st;
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}

template size_t tsqr_host_workspace<float>(int64_t, int64_t, bool);
template size_t tsqr_host_workspace<double>(int64_t, int64_t, bool);
template tsqr_status tsqr_host<float>(int64_t, int64_t, const float*, int64_t, float*, int64_t, float*, int64_t,
                                      void*, size_t, bool, cudaStream_t);
template tsqr_status tsqr_host<double>(int64_t, int64_t, const double*, int64_t, double*, int64_t, double*,
                                       int64_t, void*, size_t, bool, cudaStream_t);

// ---------------------------------------------------------------------------
// R <- R2 R (both upper triangular), for the reorthogonalisation pass of
// tsqr_*_ex.  One CTA: both factors are read into shared memory first, so R
// may be overwritten; thread (i, j) forms sum_{k=i}^{j} R2(i,k) R(k,j).
// ---------------------------------------------------------------------------
namespace {

template <typename T, int NMAX>
__global__ void upper_product_kernel(int n, const T* __restrict__ R2, int64_t ld2, T* R, int64_t ldr) {
    __shared__ T a[NMAX][NMAX + 1], b[NMAX][NMAX + 1];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        a[i][j] = R2[i + j * ld2];
        b[i][j] = R[i + j * ldr];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        T s = T(0);
        for (int k = i; k <= j; ++k) s += a[i][k] * b[k][j];
        R[i + j * ldr] = (i <= j) ? s : T(0);
    }
}

}  // namespace

template <typename T>
tsqr_status upper_product(int n, const T* R2, int64_t ld2, T* R, int64_t ldr, cudaStream_t s) {
    constexpr int NMAX = sizeof(T) == 4 ? 64 : 32;
    if (n < 1 || n > NMAX) return TSQR_ERR_UNSUPPORTED;
    upper_product_kernel<T, NMAX><<<1, 256, 0, s>>>(n, R2, ld2, R, ldr);
    log_launch(kTagTc + 902, s);
    return cudaGetLastError() == cudaSuccess ? TSQR_OK : TSQR_ERR_CUDA;
}
template tsqr_status upper_product<float>(int, const float*, int64_t, float*, int64_t, cudaStream_t);
template tsqr_status upper_product<double>(int, const double*, int64_t, double*, int64_t, cudaStream_t);

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
    if (buf[dev]) {
        // a cudaDeviceReset since the allocation invalidates it: allocate again
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, buf[dev]) != cudaSuccess || at.type != cudaMemoryTypeDevice) {
            (void)cudaGetLastError();
            buf[dev] = nullptr;
            cap[dev] = 0;
        }
    }
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
