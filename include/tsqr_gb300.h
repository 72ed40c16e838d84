/*
 * tsqr_gb300.h -- C ABI of the GB300 tall-skinny QR library.
 *
 * Every entry point takes plain device pointers, sizes and a stream handle
 * (a cudaStream_t passed as void*; NULL = the legacy default stream, where
 * the reference launches).  Matrices are column-major, as in the reference
 * (lda >= m, A[i + j*lda]).  On success A is overwritten by the thin Q
 * (m x n) and R (n x n, ldr) is fully written, zeros below the diagonal
 * included.  Calls are asynchronous on `stream`; they never assert, never
 * print and never exit: every failure comes back as a tsqr_status.
 *
 * Reference interfaces these replace (dajunHuang/tsqr):
 *   template<T> void tsqr(int m,int n,T*A,int lda,T*R,int ldr,T*d_work,int ldwork)
 *       TallShinnyQR.h:86-87, instantiated for float/double at :150-153
 *   template<T> void qr(int m,int n,T*A,int lda,T*R,int ldr,T*d_work,int ldwork)
 *       block_QR.h:72-73, instantiated for float/double at :96-99
 * The reference returns void, asserts on bad sizes (TallShinnyQR.h:92-93,
 * :109, :129; block_QR.h:78-79) and prints "not supported size" then returns
 * (TallShinnyQR.h:100-103); here those become TSQR_ERR_INVALID_ARG and
 * TSQR_ERR_UNSUPPORTED.
 */
#ifndef TSQR_GB300_H
#define TSQR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tsqr_status {
    TSQR_OK = 0,
    TSQR_ERR_INVALID_ARG = 1,   /* bad m, n, lda, ldr, null pointer, m < n  */
    TSQR_ERR_UNSUPPORTED = 2,   /* size or option the library does not cover */
    TSQR_ERR_WORKSPACE = 3,     /* workspace pointer null or too small      */
    TSQR_ERR_CUDA = 4,          /* a CUDA runtime call or launch failed     */
    TSQR_ERR_NO_DEVICE = 5      /* no CUDA device / wrong architecture      */
} tsqr_status;

/* Arithmetic of the bulk reflector applications. */
typedef enum tsqr_precision {
    TSQR_PRECISION_PLAIN = 0,   /* working precision on CUDA cores (FP32 or FP64) */
    TSQR_PRECISION_TF32X3 = 1,  /* FP32 entry points only: tcgen05 TF32 hi/lo
                                   3-product split, FP32 accumulation in TMEM  */
    TSQR_PRECISION_BF16X3 = 2   /* qr_s_ex only: its GEMMs on tcgen05 with BF16
                                   hi/lo 3-product splits (about 2^-16 relative
                                   per product), FP32 accumulation in TMEM; its
                                   TSQR panels run TF32X3.  tsqr_* entry points
                                   return TSQR_ERR_UNSUPPORTED                 */
} tsqr_precision;

/* Algorithm of qr_*_ex. */
typedef enum tsqr_qr_algorithm {
    TSQR_QR_BLOCK_GS = 0,       /* the reference's recursive block Gram-Schmidt
                                   (block_QR.h:72-95); orthogonality degrades
                                   with the condition number unless reorth   */
    TSQR_QR_HOUSEHOLDER = 1     /* blocked Householder: TSQR panels, Householder
                                   vectors reconstructed from each panel's Q,
                                   compact-WY trailing updates; orthogonal to
                                   working precision for any condition number.
                                   panel <= 32; reorth is ignored            */
} tsqr_qr_algorithm;

typedef struct tsqr_opts {
    int precision;    /* tsqr_precision; ignored (always PLAIN) for FP64    */
    int reorth;       /* 1 = one reorthogonalisation pass.  qr: a second
                         Gram-Schmidt projection (CGS2).  tsqr_*_ex: a second
                         TSQR of the computed Q in the same form, Q <- Q2 and
                         R <- R2 R1 (the workspace grows by n x n elements) */
    int panel;        /* qr only: panel width at which recursion stops, 0 = 32
                         (the reference's N_B, block_QR.h:5)                */
    int algorithm;    /* qr only: tsqr_qr_algorithm, 0 = the reference's    */
    int fp64_scalars; /* tsqr_s_ex with TF32X3 only: 1 = each column's
                         Householder norm, beta and tau computed in FP64
                         (the tile stays FP32)                              */
    int fp64_root;    /* tsqr_s_ex with TF32X3 only, n <= 32: 1 = the root of
                         the reduction tree (at most one tile of stacked R
                         factors) factored in FP64                          */
    int reserved[2];  /* must be zero                                       */
} tsqr_opts;

/* Workspace bytes an ex call needs for an m x n problem of element size
 * elem_bytes (4 or 8).  Returns 0 for sizes the library rejects. */
size_t tsqr_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts);
size_t qr_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts);

/* TSQR: replaces tsqr<float>/tsqr<double> (TallShinnyQR.h:86-153).
 * Any n >= 1 up to 64 (FP32) or 32 (FP64), any m >= n. */
tsqr_status tsqr_s_ex(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr,
                      void* work, size_t work_bytes, const tsqr_opts* opts, void* stream);
tsqr_status tsqr_d_ex(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr,
                      void* work, size_t work_bytes, const tsqr_opts* opts, void* stream);

/* Status of a call (TF32X3: tsqr_s_ex, tsqr_s_host, qr_s_ex)
 * after it has completed: the tcgen05 kernels bound every wait on their
 * mbarriers; one that runs out stops the kernel and sets a status word in
 * the first 4 bytes of the call's workspace.  Returns TSQR_OK, or
 * TSQR_ERR_CUDA when that word is set (the results are then incomplete).
 * PLAIN TSQR calls (tsqr_*_ex, tsqr_*_factor, tsqr_*_host) keep such a word
 * too, for the bounded wait of their TMA-fed tile factor.  Reads 4 bytes
 * with a synchronous copy. */
tsqr_status tsqr_workspace_check(const void* work);

/* TSQR of a matrix in host memory, with Q and R returned to host memory:
 * the call a program makes when its data are not on the GPU yet (the
 * reference's driver copies A to the device before tsqr<T>,
 * test_tsqr.cu:47-52).  Level 0 of the tree is cut into chunks of tiles; the
 * host-to-device copy of each chunk overlaps the factorisation of the
 * previous one, and the device-to-host copy of each chunk of Q overlaps the
 * Q assembly of the next, on a copy stream of the call's own.  Use pinned host
 * memory (cudaHostAlloc / cudaHostRegister) for the copies to overlap.
 * A (m x n, lda) is only read; Q (m x n, ldq) and R (n x n, ldr) are written.
 * work: device memory of tsqr_host_workspace_bytes bytes (a device copy of
 * A and the tree).  Asynchronous: the results are complete when `stream`
 * is.  precision PLAIN or TF32X3 (FP32 only). */
size_t tsqr_host_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts);
tsqr_status tsqr_s_host(int64_t m, int64_t n, const float* A, int64_t lda, float* Q, int64_t ldq,
                        float* R, int64_t ldr, void* work, size_t work_bytes, const tsqr_opts* opts,
                        void* stream);
tsqr_status tsqr_d_host(int64_t m, int64_t n, const double* A, int64_t lda, double* Q, int64_t ldq,
                        double* R, int64_t ldr, void* work, size_t work_bytes, const tsqr_opts* opts,
                        void* stream);

/* Recursive blocked QR: replaces qr<float>/qr<double> (block_QR.h:72-99):
 * qr(A1); R12 = A1^T A2; A2 -= A1 R12; qr(A2), TSQR panels at the leaves. */
tsqr_status qr_s_ex(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr,
                    void* work, size_t work_bytes, const tsqr_opts* opts, void* stream);
tsqr_status qr_d_ex(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr,
                    void* work, size_t work_bytes, const tsqr_opts* opts, void* stream);

/* Reference-signature forms (TallShinnyQR.h:87, block_QR.h:73): int sizes,
 * the caller's d_work of ldwork*n elements, legacy default stream, PLAIN
 * precision.  When d_work is smaller than the workspace this library needs,
 * a per-device buffer cached inside the library is used instead. */
tsqr_status tsqr_float(int m, int n, float* A, int lda, float* R, int ldr, float* d_work, int ldwork);
tsqr_status tsqr_double(int m, int n, double* A, int lda, double* R, int ldr, double* d_work, int ldwork);
tsqr_status qr_float(int m, int n, float* A, int lda, float* R, int ldr, float* d_work, int ldwork);
tsqr_status qr_double(int m, int n, double* A, int lda, double* R, int ldr, double* d_work, int ldwork);

/* Batched TSQR: `count` independent problems of uneven heights m[i] and
 * widths n[i] (FP32, n[i] <= 64).  The problems are grouped by (width class,
 * tile configuration); each group takes one factor launch per tree level
 * and one apply launch per level, persistent CTAs walking the group's tiles
 * from a per-problem table passed by value -- no host-to-device copy and no
 * allocation, so the whole call can be captured into one CUDA graph.  The
 * pointer/size arrays are HOST arrays; A[i], R[i] are device pointers.  No
 * counterpart in the reference (which factors one matrix per call). */
size_t tsqr_batched_workspace_bytes(int count, const int64_t* m, const int64_t* n);
tsqr_status tsqr_batched_s(int count, float* const* A, const int64_t* m, const int64_t* n,
                           const int64_t* lda, float* const* R, const int64_t* ldr,
                           void* work, size_t work_bytes, const tsqr_opts* opts, void* stream);

/* Autotuner of the batched form.  Each width class (0: n <= 8, 1: n <= 16,
 * 2: n <= 32, 3: n <= 64) has candidate tile configurations (candidate 0 is
 * the single-problem path's tile height, candidate 1 half of it), chosen per
 * height bucket (0: m < 8192, 1: m < 65536, 2: m >= 65536) by a
 * process-wide table that tsqr_batched_s reads once per call.
 * tsqr_batched_tune_s times every candidate of each (class, bucket) present
 * in the given shapes, on synthetic matrices of those shapes (reps timed
 * runs after one warm-up), and keeps the fastest.  It allocates its own
 * scratch, synchronizes, and must not run concurrently with batched calls.
 * The workspace size of tsqr_batched_workspace_bytes holds for every choice. */
tsqr_status tsqr_batched_tune_s(int count, const int64_t* m, const int64_t* n, int reps, void* stream);
int tsqr_batched_choice(int width_class, int height_bucket);         /* -1 on bad arguments */
int tsqr_batched_candidate_rows(int width_class, int candidate);     /* tile height, -1 on bad arguments */
tsqr_status tsqr_batched_set_choice(int width_class, int height_bucket, int candidate);

/* FP32 TSQR that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: frameworks that have already
 * reserved nearly all device memory for their own pool, programs with a
 * memory budget set at start-up, callers that cannot afford the device-wide
 * synchronisation a cudaFree may cause, and callers of the reference's
 * interface whose d_work cannot grow.  Same arithmetic and results as
 * tsqr_s_ex with PLAIN precision; the tree workspace lives in one static
 * device array of TSQR_NOALLOC_SCRATCH_BYTES inside the library, held by
 * every GPU that loads the library until exit.  Problems whose workspace
 * (tsqr_workspace_bytes) exceeds that size return TSQR_ERR_WORKSPACE
 * without launching (with n = 32, up to about 1.9 million rows fit).
 * The first call on a device looks up the array's device address with that
 * device current; make it before any stream capture.  Later calls repeat the
 * lookup whenever their stream is not capturing (after a cudaDeviceReset
 * the array may sit at a new address).  All calls on a
 * device share the array: calls that overlap on the GPU race, so the caller
 * must order them (one stream, or explicit synchronisation). */
#define TSQR_NOALLOC_SCRATCH_BYTES (16u << 20)
tsqr_status tsqr_s_noalloc(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* stream);

/* Instrumentation (no counterpart in the reference): runs tsqr (kind 0) or
 * qr (kind 1) exactly as the _ex entry points do, recording a CUDA event on
 * `stream` before the first and after every kernel launch; synchronizes on
 * the last event and writes each launch's device time in ms and its tag
 * (kind*1000 + tree level; kinds 1 factor, 2 apply, 3-6 blocked-QR GEMM
 * steps, 7 tensor-core kernels, 8 batched) to launch_ms / launch_tag. */
tsqr_status tsqr_profile(int kind, int elem_bytes, int64_t m, int64_t n, void* A, int64_t lda, void* R,
                         int64_t ldr, void* work, size_t work_bytes, const tsqr_opts* opts, void* stream,
                         float* launch_ms, int* launch_tag, int max_launch, int* n_launch);

/* Implicit-Q form (no counterpart in the reference, which always forms the
 * explicit thin Q, kernelQR.h:224-290).
 * tsqr_*_factor runs the up-sweep only.  A keeps level 0 of the compact-WY
 *   tree (Householder vectors below each tile's diagonal, T in its top
 *   block), `work` (tsqr_workspace_bytes, PLAIN precision) keeps the upper
 *   levels, and R is written as by tsqr_*_ex.  Leave A and work unchanged
 *   while the factorisation is in use.  PLAIN precision only.
 * tsqr_*_apply_qt: D (n x k, ldd >= n) = Q^T C for C (m x k, ldc >= m),
 *   walking the same tree upwards; C is only read.  cwork holds the stacked
 *   intermediate levels: tsqr_apply_qt_workspace_bytes(m, n, k, elem_bytes)
 *   bytes.  n <= 64 (FP32) / 32 (FP64).
 * tsqr_*_form_q runs the down-sweep: A becomes the explicit thin Q, exactly
 *   as tsqr_*_ex leaves it; the tree in A is consumed. */
tsqr_status tsqr_s_factor(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                          size_t work_bytes, const tsqr_opts* opts, void* stream);
tsqr_status tsqr_d_factor(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr, void* work,
                          size_t work_bytes, const tsqr_opts* opts, void* stream);
size_t tsqr_apply_qt_workspace_bytes(int64_t m, int64_t n, int64_t k, int elem_bytes);
tsqr_status tsqr_s_apply_qt(int64_t m, int64_t n, const float* V, int64_t ldv, const void* work, size_t work_bytes,
                            int64_t k, const float* C, int64_t ldc, float* D, int64_t ldd, void* cwork,
                            size_t cwork_bytes, void* stream);
tsqr_status tsqr_d_apply_qt(int64_t m, int64_t n, const double* V, int64_t ldv, const void* work, size_t work_bytes,
                            int64_t k, const double* C, int64_t ldc, double* D, int64_t ldd, void* cwork,
                            size_t cwork_bytes, void* stream);
tsqr_status tsqr_s_form_q(int64_t m, int64_t n, float* A, int64_t lda, void* work, size_t work_bytes, void* stream);
tsqr_status tsqr_d_form_q(int64_t m, int64_t n, double* A, int64_t lda, void* work, size_t work_bytes, void* stream);

/* Accuracy of a thin QR, computed on the GPU in FP64.  Replaces the
 * reference's host accuracy check check_QR_accuracy (utils.h:317-455), whose
 * cuSOLVER gesvd workspace overflows int past m = 46,340.  A is the original
 * m x n matrix, Q the thin Q (ldq >= m) and R the n x n factor (ldr >= n),
 * device pointers of element size elem_bytes (4 or 8).  The element gate is
 * the reference's all_close (utils.h:148-174; the reference passes atol 1e-4,
 * rtol 1e-5): |(QR)_ij - A_ij| <= max(atol, rtol |A_ij|), NaN fails, and the
 * first failure is the first in column-major order, as there.  The spectral
 * figures are the two the reference prints (utils.h:380).  Synchronizes on
 * `stream`; the result is written to host memory. */
typedef struct tsqr_check_result {
    double backward_fro;   /* ||A - QR||_F / ||A||_F                 */
    double orth_fro;       /* ||Q^T Q - I||_F                        */
    double backward_2;     /* ||A - QR||_2 / ||A||_2                 */
    double orth_2;         /* ||I - Q^T Q||_2 / n                    */
    int64_t gate_failures; /* elements outside the gate              */
    int64_t first_row;     /* first failing element, -1 if none      */
    int64_t first_col;
    double first_value;    /* (QR) at the first failure              */
    double first_ref;      /* A at the first failure                 */
} tsqr_check_result;

/* Workspace bytes of tsqr_check: an m x n FP64 residual, the Gram partials
 * (ceil(m / 4096) x n x n doubles) and three n x n Gram matrices. */
size_t tsqr_check_workspace_bytes(int64_t m, int64_t n);
tsqr_status tsqr_check(int elem_bytes, int64_t m, int64_t n, const void* A, int64_t lda, const void* Q, int64_t ldq,
                       const void* R, int64_t ldr, double atol, double rtol, void* work, size_t work_bytes,
                       void* stream, tsqr_check_result* out);

/* Human-readable text of a status; never NULL. */
const char* tsqr_status_string(tsqr_status s);

/* Library version, e.g. "0.1.0". */
const char* tsqr_version(void);

/* Test hook for the failure path of the kernels that wait on an mbarrier
 * (no counterpart in the reference, whose grid barrier spins without a
 * limit, kernelQR.h:374).  Sets how many times the kernels of later calls
 * poll an mbarrier before giving up: the tcgen05 kernels (tc_apply_tiles,
 * tc_gemm_kernel) for their MMAs, and the TMA-staged tile factor for its
 * tile.  0 makes the first wait of every such kernel give up at once, so
 * the call's status word is set and tsqr_workspace_check reports
 * TSQR_ERR_CUDA.  The waits that let in-flight MMAs retire before TMEM is
 * freed, or in-flight copies land before a CTA exits, always keep the full
 * limit.  polls < 0 restores the default (2^24 polls, seconds).
 * Process-wide; for tests only. */
tsqr_status tsqr_debug_set_wait_limit(int polls);

#ifdef __cplusplus
}
#endif

#endif /* TSQR_GB300_H */
