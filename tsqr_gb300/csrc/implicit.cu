// implicit.cu -- the implicit-Q form of TSQR: factor once, then apply Q^T
// (tsqr_*_factor, tsqr_*_apply_qt, tsqr_*_form_q).
//
// The reference always forms the explicit thin Q (kernelQR.h:224-290 and
// the down-sweep, kernelQR.h:397-492).  A caller that only needs Q^T C (a
// least-squares solve: x = R^-1 Q^T b) can stop after the up-sweep: the
// tree of compact-WY factors it leaves (level 0 in A, the upper levels in
// the workspace) represents Q = Q_0 Q_1 ... Q_L, Q_l = blockdiag over the
// level's tiles of H_t [I_n; 0] with H_t = I - V_t T_t V_t^T.  Then
//   Q^T C = Q_L^T ... Q_1^T Q_0^T C,
// and Q_0^T C takes, per tile t, the top n rows of H_t^T C_t:
//   C_t,top - V_t,top Z_t,   Z_t = T_t^T (V_t^T C_t),
// which stack (tiles x n rows) into the next level's C.  The root writes the
// n x k result.  C is read once; only the n x k stacks of the upper levels
// are written -- against the explicit path's full Q (m x n written, then
// read again by the caller's Q^T C product).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/tsqr_gb300.h"
#include "common.cuh"
#include "internal.h"

namespace tsqr {
namespace {

constexpr int kKB = 32;   // columns of C per CTA
constexpr int kCH = 64;   // tile rows staged per chunk
constexpr int kNT = 256;  // threads per CTA

template <typename T, int NMAX>
struct QtSmem {
    static constexpr int SW = NMAX;  // V chunk row stride; 4-element groups are XOR-swizzled by row
    T Vs[kCH][SW];                   // masked V rows of the chunk
    T Cs[kCH][kKB + 1];              // C rows of the chunk
    T Tr[NMAX][NMAX + 1];            // the tile's raw top block (T above, V_top below the diagonal)
    T Ys[NMAX][kKB + 1];             // Y = V^T C, then Z = T^T Y
    T Zs[NMAX][kKB + 1];
};

// Column group g (4 consecutive columns) of V row r sits at group g ^ (r & 7):
// the staging stores of 32 consecutive rows then spread over 8 bank groups,
// and a row's 4 columns stay one 16-byte (float) / two 8-byte (double) load.
template <int NMAX>
__device__ __forceinline__ int vcol(int r, int j) {
    static_assert(NMAX % 32 == 0, "V groups must cover 8 swizzle positions");
    return ((((j >> 2) ^ (r & 7))) << 2) | (j & 3);
}

// four consecutive elements from a 16-byte aligned shared address
__device__ __forceinline__ void load4(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
}
__device__ __forceinline__ void load4(const double* p, double (&v)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x, v[1] = a.y, v[2] = b.x, v[3] = b.y;
}

template <typename T, int NMAX>
struct QtParams {
    const T* M;   // level matrix: V below the diagonal, T in each tile's top block
    int64_t ld, h, ntiles;
    int rows;     // tile height B
    int n;
    const T* C;   // this level's C (h x k)
    int64_t ldc;
    T* out;       // next level's C (rows t*n + j), or the n x k result at the root
    int64_t ldo;
    int64_t k;
};

template <typename T, int NMAX>
__global__ void __launch_bounds__(kNT) apply_qt_tiles(QtParams<T, NMAX> p) {
    pdl_begin();
    extern __shared__ __align__(16) unsigned char qt_smem_raw[];
    QtSmem<T, NMAX>& S = *reinterpret_cast<QtSmem<T, NMAX>*>(qt_smem_raw);
    constexpr int JPT = NMAX / 8;  // outputs j per thread (8 warps x JPT = NMAX)
    const int tid = threadIdx.x;
    const int c = tid % 32, j0 = (tid / 32) * JPT;
    const int n = p.n;
    const int64_t kblocks = (p.k + kKB - 1) / kKB;
    for (int64_t w = blockIdx.x; w < p.ntiles * kblocks; w += gridDim.x) {
        const int64_t t = w / kblocks;
        const int64_t c0 = (w % kblocks) * kKB;
        const int64_t row0 = t * p.rows;
        const int ht = (int)((p.h - row0) < p.rows ? (p.h - row0) : p.rows);
        const T* tile = p.M + row0;
        const T* ct = p.C + row0;

        // ---- Y = V^T C over the tile's rows, chunk by chunk ---------------
        T acc[JPT];
#pragma unroll
        for (int s = 0; s < JPT; ++s) acc[s] = T(0);
        for (int r0 = 0; r0 < ht; r0 += kCH) {
            constexpr int PV = kCH * NMAX / kNT, PC = kCH * kKB / kNT;
            T gv[PV], gc[PC];
#pragma unroll
            for (int q = 0; q < PV; ++q) {
                const int e = tid + kNT * q;
                const int r = e % kCH, j = e / kCH;
                const int rr = r0 + r;
                gv[q] = (rr < ht && j < n && rr > j) ? tile[rr + (int64_t)j * p.ld] : T(0);
            }
#pragma unroll
            for (int q = 0; q < PC; ++q) {
                const int e = tid + kNT * q;
                const int r = e % kCH, cc = e / kCH;
                const int rr = r0 + r;
                gc[q] = (rr < ht && c0 + cc < p.k) ? ct[rr + (c0 + cc) * p.ldc] : T(0);
            }
#pragma unroll
            for (int q = 0; q < PV; ++q) {
                const int e = tid + kNT * q;
                const int r = e % kCH, j = e / kCH;
                const int rr = r0 + r;
                S.Vs[r][vcol<NMAX>(r, j)] = (rr == j && j < n && rr < ht) ? T(1) : gv[q];
            }
#pragma unroll
            for (int q = 0; q < PC; ++q) {
                const int e = tid + kNT * q;
                S.Cs[e % kCH][e / kCH] = gc[q];
            }
            __syncthreads();
            const int rmax = min(kCH, ht - r0);
            for (int r = 0; r < rmax; ++r) {
                const T cv = S.Cs[r][c];
#pragma unroll
                for (int g = 0; g < JPT; g += 4) {
                    T v[4];
                    load4(&S.Vs[r][vcol<NMAX>(r, j0 + g)], v);
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[g + e] = fma(v[e], cv, acc[g + e]);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int s = 0; s < JPT; ++s) S.Ys[j0 + s][c] = acc[s];
        // the tile's top block (rows past the tile end read as zero)
        for (int e = tid; e < NMAX * NMAX; e += kNT) {
            const int i = e % NMAX, j = e / NMAX;
            S.Tr[i][j] = (i < ht && i < n && j < n) ? tile[i + (int64_t)j * p.ld] : T(0);
        }
        __syncthreads();

        // ---- Z = T^T Y (T upper triangular: Z_j = sum_{i <= j} T(i,j) Y_i) --
#pragma unroll
        for (int s = 0; s < JPT; ++s) {
            const int j = j0 + s;
            T z = T(0);
            for (int i = 0; i <= j && i < n; ++i) z = fma(S.Tr[i][j], S.Ys[i][c], z);
            S.Zs[j][c] = z;
        }
        __syncthreads();

        // ---- top n rows of C - V Z (V_top unit lower triangular) ------------
#pragma unroll
        for (int s = 0; s < JPT; ++s) {
            const int j = j0 + s;
            if (j < n && c0 + c < p.k) {
                T v = (j < ht) ? ct[j + (c0 + c) * p.ldc] : T(0);
                v -= S.Zs[j][c];
                for (int i = 0; i < j; ++i) v = fma(-S.Tr[j][i], S.Zs[i][c], v);
                p.out[t * n + j + (c0 + c) * p.ldo] = v;
            }
        }
        __syncthreads();  // the shared buffers are reused by the next work item
    }
}

// Sum of v[0..31] over the warp, scattered: lane l returns the total of
// index l.  Five halving rounds (16 + 8 + 4 + 2 + 1 shuffles): in the round
// of offset o a lane keeps the half of its live values selected by bit o of
// its lane index and adds the partner's copy of that half.
template <typename T>
__device__ __forceinline__ T warp_reduce_scatter32(T (&v)[32], int lane) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const T send = upper ? v[i] : v[i + o];
            const T keep = upper ? v[i + o] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

// Q^T c for one column c of C (k small): thread rows read V and c directly
// from global memory (coalesced along each column), Y = V^T c accumulates in
// registers and is reduced across the CTA (warp reduce-scatter, then the
// warps' partials through shared memory).  No staging of V, so the kernel
// streams the level at close to the memory rate.  Tile heights up to 1024.
template <typename T, int NMAX>
__global__ void __launch_bounds__(kNT) apply_qt_column(QtParams<T, NMAX> p, int64_t col) {
    pdl_begin();
    constexpr int NW = kNT / 32;
    __shared__ T ys[NW][NMAX];
    __shared__ T yv[NMAX], zv[NMAX];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n = p.n;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
        const int64_t row0 = t * p.rows;
        const int ht = (int)((p.h - row0) < p.rows ? (p.h - row0) : p.rows);
        const T* tile = p.M + row0;
        const T* ct = p.C + row0 + col * p.ldc;
        T acc[NMAX];
#pragma unroll
        for (int j = 0; j < NMAX; ++j) acc[j] = T(0);
#pragma unroll 1
        for (int i = 0; i < 4; ++i) {
            const int r = tid + kNT * i;
            if (r < ht) {
                const T cr = ct[r];
                T v[NMAX];
#pragma unroll
                for (int j = 0; j < NMAX; ++j)
                    v[j] = (j < n && r > j) ? tile[r + (int64_t)j * p.ld] : ((j < n && r == j) ? T(1) : T(0));
#pragma unroll
                for (int j = 0; j < NMAX; ++j) acc[j] = fma(v[j], cr, acc[j]);
            }
        }
#pragma unroll
        for (int h = 0; h < NMAX; h += 32) {
            T part[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) part[j] = acc[h + j];
            ys[warp][h + lane] = warp_reduce_scatter32(part, lane);
        }
        __syncthreads();
        if (tid < NMAX) {
            T y = T(0);
#pragma unroll
            for (int w = 0; w < NW; ++w) y += ys[w][tid];
            yv[tid] = y;
        }
        __syncthreads();
        // Z = T^T Y, then the top n rows of c - V Z
        if (tid < n) {
            const int j = tid;
            T z = T(0);
            for (int i = 0; i <= j; ++i) z = fma((i < ht) ? tile[i + (int64_t)j * p.ld] : T(0), yv[i], z);
            zv[j] = z;
        }
        __syncthreads();
        if (tid < n) {
            const int j = tid;
            T v = ((j < ht) ? ct[j] : T(0)) - zv[j];
            for (int i = 0; i < j; ++i) v = fma((j < ht) ? -tile[j + (int64_t)i * p.ld] : T(0), zv[i], v);
            p.out[t * n + j + col * p.ldo] = v;
        }
        __syncthreads();  // ys / yv / zv are reused by the next tile
    }
}

template <typename T, int NMAX>
cudaError_t launch_apply_qt(const QtParams<T, NMAX>& p, cudaStream_t s) {
    if (p.k <= 2 && p.rows <= 4 * kNT) {
        // one or two columns: one streaming pass per column (about 0.28 ms
        // each at 4,194,304 x 32, against about 0.75 ms for the blocked
        // kernel at any k up to 32)
        const int sms = device_sm_count();
        const int grid = (int)std::min<int64_t>(p.ntiles, (int64_t)sms * 8);
        for (int64_t c = 0; c < p.k; ++c) launch_pdl(apply_qt_column<T, NMAX>, dim3(grid), dim3(kNT), 0, s, p, c);
        return cudaGetLastError();
    }
    constexpr size_t smem = sizeof(QtSmem<T, NMAX>);
    // a failure shows here on the device's first call, and in the launch
    // error of every later one
    cudaError_t attr = cudaSuccess;
    static PerDeviceOnce attr_once;
    attr_once.run([&] {
        attr = cudaFuncSetAttribute(apply_qt_tiles<T, NMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (attr != cudaSuccess) return attr;
    const int64_t items = p.ntiles * ((p.k + kKB - 1) / kKB);
    const int grid = (int)std::min<int64_t>(items, 1 << 20);
    launch_pdl(apply_qt_tiles<T, NMAX>, dim3(grid), dim3(kNT), smem, s, p);
    return cudaGetLastError();
}

// Stacked C of levels 1.. in the apply workspace, 256-byte aligned.
template <typename T>
size_t qt_layout(const std::vector<TreeLevel<T>>& lv, int64_t k, std::vector<size_t>* off) {
    size_t o = 0;
    if (off) off->assign(lv.size(), 0);
    for (size_t l = 1; l < lv.size(); ++l) {
        if (off) (*off)[l] = o;
        o += (size_t)((lv[l].ld * k * (int64_t)sizeof(T) + 255) / 256 * 256);
    }
    return o;
}

template <typename T>
int qt_nmax(int64_t n) {
    if (n <= 32) return 32;
    if (sizeof(T) == 4 && n <= 64) return 64;
    return 0;
}

template <typename T>
tsqr_status apply_qt_impl(int64_t m, int64_t n, const T* V, int64_t ldv, const void* work, size_t work_bytes,
                          int64_t k, const T* C, int64_t ldc, T* D, int64_t ldd, void* cwork, size_t cwork_bytes,
                          cudaStream_t s) {
    if (m < 1 || n < 1 || m < n || k < 1 || !V || !C || !D || ldv < m || ldc < m || ldd < n)
        return TSQR_ERR_INVALID_ARG;
    const int nmax = qt_nmax<T>(n);
    if (!nmax) return TSQR_ERR_UNSUPPORTED;
    std::vector<TreeLevel<T>> lv;
    tsqr_status st = tsqr_plain_tree<T>(m, n, V, ldv, work, work_bytes, &lv);
    if (st != TSQR_OK) return st;
    std::vector<size_t> off;
    const size_t need = qt_layout<T>(lv, k, &off);
    if (need > 0 && (!cwork || cwork_bytes < need)) return TSQR_ERR_WORKSPACE;
    const T* cin = C;
    int64_t ldin = ldc;
    for (size_t l = 0; l < lv.size(); ++l) {
        const bool root = (l + 1 == lv.size());
        T* out = root ? D : reinterpret_cast<T*>(static_cast<char*>(cwork) + off[l + 1]);
        const int64_t ldo = root ? ldd : lv[l + 1].ld;
        cudaError_t e;
        if (nmax == 32) {
            QtParams<T, 32> p{lv[l].M, lv[l].ld, lv[l].h, lv[l].ntiles, lv[l].rows, (int)n, cin, ldin, out, ldo, k};
            e = launch_apply_qt<T, 32>(p, s);
        } else {
            QtParams<T, 64> p{lv[l].M, lv[l].ld, lv[l].h, lv[l].ntiles, lv[l].rows, (int)n, cin, ldin, out, ldo, k};
            e = launch_apply_qt<T, 64>(p, s);
        }
        if (e != cudaSuccess) return TSQR_ERR_CUDA;
        log_launch(kTagApplyQt + (int)l, s);
        cin = out;
        ldin = ldo;
    }
    return TSQR_OK;
}

template <typename T>
size_t apply_qt_workspace(int64_t m, int64_t n, int64_t k) {
    if (m < 1 || n < 1 || m < n || k < 1 || !qt_nmax<T>(n)) return 0;
    std::vector<TreeLevel<T>> lv;
    // the layout depends on sizes only: plan it on a dummy base
    const size_t wb = tsqr_plain_workspace<T>(m, n);
    if (tsqr_plain_tree<T>(m, n, reinterpret_cast<const T*>(256), m, reinterpret_cast<const void*>(256), wb, &lv) !=
        TSQR_OK)
        return 0;
    const size_t b = qt_layout<T>(lv, k, nullptr);
    return b ? b : 256;
}

}  // namespace
}  // namespace tsqr

extern "C" {

size_t tsqr_apply_qt_workspace_bytes(int64_t m, int64_t n, int64_t k, int elem_bytes) {
    if (elem_bytes == 4) return tsqr::apply_qt_workspace<float>(m, n, k);
    if (elem_bytes == 8) return tsqr::apply_qt_workspace<double>(m, n, k);
    return 0;
}

tsqr_status tsqr_s_apply_qt(int64_t m, int64_t n, const float* V, int64_t ldv, const void* work, size_t work_bytes,
                            int64_t k, const float* C, int64_t ldc, float* D, int64_t ldd, void* cwork,
                            size_t cwork_bytes, void* stream) {
    return tsqr::apply_qt_impl<float>(m, n, V, ldv, work, work_bytes, k, C, ldc, D, ldd, cwork, cwork_bytes,
                                      static_cast<cudaStream_t>(stream));
}

tsqr_status tsqr_d_apply_qt(int64_t m, int64_t n, const double* V, int64_t ldv, const void* work, size_t work_bytes,
                            int64_t k, const double* C, int64_t ldc, double* D, int64_t ldd, void* cwork,
                            size_t cwork_bytes, void* stream) {
    return tsqr::apply_qt_impl<double>(m, n, V, ldv, work, work_bytes, k, C, ldc, D, ldd, cwork, cwork_bytes,
                                       static_cast<cudaStream_t>(stream));
}

}  // extern "C"
