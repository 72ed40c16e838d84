// abi.cu -- extern "C" entry points of libtsqr_gb300.so.
//
// Argument checks replace the reference's host asserts and its silent
// "not supported size" return (TallShinnyQR.h:92-93, :100-103, :109, :129;
// block_QR.h:78-79): every rejected call returns a status and launches
// nothing.
#include <cuda_runtime.h>

#include "../../include/tsqr_gb300.h"
#include "internal.h"

namespace {

tsqr_opts opts_or_default(const tsqr_opts* o) {
    tsqr_opts d = {};
    return o ? *o : d;
}

template <typename T>
int max_tsqr_n() {
    return sizeof(T) == 4 ? 64 : 32;
}

template <typename T>
tsqr_status check_common(int64_t m, int64_t n, const T* A, int64_t lda, const T* R, int64_t ldr,
                         const tsqr_opts& o) {
    if (m < 1 || n < 1 || m < n) return TSQR_ERR_INVALID_ARG;
    if (lda < m || ldr < n) return TSQR_ERR_INVALID_ARG;
    if (A == nullptr || R == nullptr) return TSQR_ERR_INVALID_ARG;
    for (int i = 0; i < 2; ++i)
        if (o.reserved[i] != 0) return TSQR_ERR_INVALID_ARG;
    if (o.fp64_scalars < 0 || o.fp64_scalars > 1 || o.fp64_root < 0 || o.fp64_root > 1) return TSQR_ERR_INVALID_ARG;
    if (o.algorithm != TSQR_QR_BLOCK_GS && o.algorithm != TSQR_QR_HOUSEHOLDER) return TSQR_ERR_INVALID_ARG;
    if (o.precision < TSQR_PRECISION_PLAIN || o.precision > TSQR_PRECISION_BF16X3) return TSQR_ERR_INVALID_ARG;
    if (o.panel < 0 || o.reorth < 0 || o.reorth > 1) return TSQR_ERR_INVALID_ARG;
    return TSQR_OK;
}

constexpr size_t kAlignAbi = 256;
size_t align_up(size_t b) { return (b + kAlignAbi - 1) / kAlignAbi * kAlignAbi; }

// Workspace of tsqr_*_ex: the form's tree workspace, then (reorth) the
// second pass's n x n R.  0 for what the library does not cover.
template <typename T>
size_t tsqr_ex_workspace(int64_t m, int64_t n, const tsqr_opts& o) {
    const bool prec = sizeof(T) == 4 && o.precision == TSQR_PRECISION_TF32X3;
    if (n > max_tsqr_n<T>()) return 0;
    if (sizeof(T) == 4 && o.precision == TSQR_PRECISION_BF16X3) return 0;
    if (!prec && (o.fp64_scalars || o.fp64_root)) return 0;
    if (prec && o.fp64_root && n > 32) return 0;
    tsqr::PrecFlags f;
    f.norm64 = o.fp64_scalars != 0;
    f.root64 = o.fp64_root != 0;
    const size_t base = prec ? tsqr::tsqr_precision_workspace(m, n, f) : tsqr::tsqr_plain_workspace<T>(m, n);
    if (base == 0) return 0;
    return o.reorth ? align_up(base) + align_up((size_t)(n * n) * sizeof(T)) : base;
}

template <typename T>
tsqr_status tsqr_ex(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                    const tsqr_opts* op, void* stream) {
    const tsqr_opts o = opts_or_default(op);
    tsqr_status st = check_common<T>(m, n, A, lda, R, ldr, o);
    if (st != TSQR_OK) return st;
    if (tsqr_ex_workspace<T>(m, n, o) == 0) return TSQR_ERR_UNSUPPORTED;
    const cudaStream_t s = (cudaStream_t)stream;
    const bool prec = sizeof(T) == 4 && o.precision == TSQR_PRECISION_TF32X3;
    tsqr::PrecFlags f;
    f.norm64 = o.fp64_scalars != 0;
    f.root64 = o.fp64_root != 0;
    // one TSQR pass of the chosen form over A, its R to Rp; a second pass
    // keeps the first pass's tensor-core status
    auto pass = [&](T* Rp, int64_t ldrp, size_t bytes, bool first) -> tsqr_status {
        if (prec) {
            f.clear_status = first;
            return tsqr::tsqr_precision(m, n, reinterpret_cast<float*>(A), lda, reinterpret_cast<float*>(Rp), ldrp,
                                        work, bytes, s, f);
        }
        return tsqr::tsqr_plain<T>(m, n, A, lda, Rp, ldrp, work, bytes, s);
    };
    if (!o.reorth) return pass(R, ldr, work_bytes, true);
    // one reorthogonalisation pass: Q1 R1 = A, then Q2 R2 = Q1, so that
    // A = Q2 (R2 R1)
    const size_t need = tsqr_ex_workspace<T>(m, n, o);
    if (work == nullptr || work_bytes < need) return TSQR_ERR_WORKSPACE;
    const size_t base = need - align_up((size_t)(n * n) * sizeof(T));
    T* R2 = reinterpret_cast<T*>(reinterpret_cast<char*>(work) + base);
    st = pass(R, ldr, base, true);
    if (st != TSQR_OK) return st;
    st = pass(R2, n, base, false);
    if (st != TSQR_OK) return st;
    return tsqr::upper_product<T>((int)n, R2, n, R, ldr, s);
}

// Implicit-Q form: the up-sweep alone, and later the down-sweep alone, on
// the same tree (plain precision only).
template <typename T>
tsqr_status factor_ex(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                      const tsqr_opts* op, void* stream) {
    const tsqr_opts o = opts_or_default(op);
    tsqr_status st = check_common<T>(m, n, A, lda, R, ldr, o);
    if (st != TSQR_OK) return st;
    if (n > max_tsqr_n<T>() || o.precision != TSQR_PRECISION_PLAIN || o.reorth || o.fp64_scalars || o.fp64_root)
        return TSQR_ERR_UNSUPPORTED;
    return tsqr::tsqr_plain<T>(m, n, A, lda, R, ldr, work, work_bytes, (cudaStream_t)stream, tsqr::kPhaseUp);
}

template <typename T>
tsqr_status form_q_ex(int64_t m, int64_t n, T* A, int64_t lda, void* work, size_t work_bytes, void* stream) {
    if (m < 1 || n < 1 || m < n || lda < m || A == nullptr) return TSQR_ERR_INVALID_ARG;
    if (n > max_tsqr_n<T>()) return TSQR_ERR_UNSUPPORTED;
    return tsqr::tsqr_plain<T>(m, n, A, lda, nullptr, n, work, work_bytes, (cudaStream_t)stream, tsqr::kPhaseDown);
}

template <typename T>
tsqr_status qr_ex(int64_t m, int64_t n, T* A, int64_t lda, T* R, int64_t ldr, void* work, size_t work_bytes,
                  const tsqr_opts* op, void* stream) {
    const tsqr_opts o = opts_or_default(op);
    tsqr_status st = check_common<T>(m, n, A, lda, R, ldr, o);
    if (st != TSQR_OK) return st;
    if (o.panel > max_tsqr_n<T>() || o.fp64_scalars || o.fp64_root) return TSQR_ERR_UNSUPPORTED;
    return tsqr::qr_run<T>(m, n, A, lda, R, ldr, work, work_bytes, o, (cudaStream_t)stream);
}

// Reference-signature form: the caller's d_work (ldwork*n elements) is used
// when it is large enough, the library's cached buffer otherwise.
template <typename T, bool QR>
tsqr_status ref_form(int m, int n, T* A, int lda, T* R, int ldr, T* d_work, int ldwork) {
    tsqr_opts o = {};
    if (m < 1 || n < 1) return TSQR_ERR_INVALID_ARG;
    size_t need = QR ? tsqr::qr_workspace<T>(m, n, o) : tsqr::tsqr_plain_workspace<T>(m, n);
    if (!QR && n > max_tsqr_n<T>()) return TSQR_ERR_UNSUPPORTED;
    void* work = d_work;
    size_t have = (d_work && ldwork > 0) ? (size_t)ldwork * (size_t)n * sizeof(T) : 0;
    if (have < need) {
        tsqr_status st;
        work = tsqr::cached_workspace(need, &st);
        if (!work) return st;
        have = need;
    }
    return QR ? qr_ex<T>(m, n, A, lda, R, ldr, work, have, &o, nullptr)
              : tsqr_ex<T>(m, n, A, lda, R, ldr, work, have, &o, nullptr);
}

template <typename T>
tsqr_status tsqr_host_call(int64_t m, int64_t n, const T* A, int64_t lda, T* Q, int64_t ldq, T* R, int64_t ldr,
                           void* work, size_t work_bytes, const tsqr_opts* op, void* stream) {
    const tsqr_opts o = opts_or_default(op);
    tsqr_status st = check_common<T>(m, n, A, lda, R, ldr, o);
    if (st != TSQR_OK) return st;
    if (Q == nullptr || ldq < m) return TSQR_ERR_INVALID_ARG;
    if (n > max_tsqr_n<T>()) return TSQR_ERR_UNSUPPORTED;
    if (o.precision == TSQR_PRECISION_BF16X3 || (sizeof(T) == 8 && o.precision != TSQR_PRECISION_PLAIN) || o.reorth ||
        o.fp64_scalars || o.fp64_root)
        return TSQR_ERR_UNSUPPORTED;
    return tsqr::tsqr_host<T>(m, n, A, lda, Q, ldq, R, ldr, work, work_bytes,
                              o.precision == TSQR_PRECISION_TF32X3, (cudaStream_t)stream);
}

}  // namespace

extern "C" {

size_t tsqr_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts) {
    const tsqr_opts o = opts_or_default(opts);
    if (m < 1 || n < 1 || m < n) return 0;
    if (elem_bytes == 4) return tsqr_ex_workspace<float>(m, n, o);
    if (elem_bytes == 8) return tsqr_ex_workspace<double>(m, n, o);
    return 0;
}

tsqr_status tsqr_workspace_check(const void* work) {
    if (work == nullptr) return TSQR_ERR_INVALID_ARG;
    int word = 0;
    if (cudaMemcpy(&word, work, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return TSQR_ERR_CUDA;
    return word == 0 ? TSQR_OK : TSQR_ERR_CUDA;
}

size_t tsqr_host_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts) {
    const tsqr_opts o = opts_or_default(opts);
    if (m < 1 || n < 1 || m < n) return 0;
    const bool prec = o.precision == TSQR_PRECISION_TF32X3;
    if (elem_bytes == 4) return n <= 64 ? tsqr::tsqr_host_workspace<float>(m, n, prec) : 0;
    if (elem_bytes == 8) return (n <= 32 && !prec) ? tsqr::tsqr_host_workspace<double>(m, n, false) : 0;
    return 0;
}

tsqr_status tsqr_s_host(int64_t m, int64_t n, const float* A, int64_t lda, float* Q, int64_t ldq, float* R,
                        int64_t ldr, void* work, size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return tsqr_host_call<float>(m, n, A, lda, Q, ldq, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status tsqr_d_host(int64_t m, int64_t n, const double* A, int64_t lda, double* Q, int64_t ldq, double* R,
                        int64_t ldr, void* work, size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return tsqr_host_call<double>(m, n, A, lda, Q, ldq, R, ldr, work, work_bytes, opts, stream);
}

size_t qr_workspace_bytes(int64_t m, int64_t n, int elem_bytes, const tsqr_opts* opts) {
    const tsqr_opts o = opts_or_default(opts);
    if (m < 1 || n < 1 || m < n) return 0;
    if (elem_bytes == 4) return tsqr::qr_workspace<float>(m, n, o);
    if (elem_bytes == 8) return tsqr::qr_workspace<double>(m, n, o);
    return 0;
}

tsqr_status tsqr_s_ex(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                      size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return tsqr_ex<float>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status tsqr_d_ex(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr, void* work,
                      size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return tsqr_ex<double>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status tsqr_s_factor(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                          size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return factor_ex<float>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status tsqr_d_factor(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr, void* work,
                          size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return factor_ex<double>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status tsqr_s_form_q(int64_t m, int64_t n, float* A, int64_t lda, void* work, size_t work_bytes, void* stream) {
    return form_q_ex<float>(m, n, A, lda, work, work_bytes, stream);
}
tsqr_status tsqr_d_form_q(int64_t m, int64_t n, double* A, int64_t lda, void* work, size_t work_bytes,
                          void* stream) {
    return form_q_ex<double>(m, n, A, lda, work, work_bytes, stream);
}
tsqr_status qr_s_ex(int64_t m, int64_t n, float* A, int64_t lda, float* R, int64_t ldr, void* work,
                    size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return qr_ex<float>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}
tsqr_status qr_d_ex(int64_t m, int64_t n, double* A, int64_t lda, double* R, int64_t ldr, void* work,
                    size_t work_bytes, const tsqr_opts* opts, void* stream) {
    return qr_ex<double>(m, n, A, lda, R, ldr, work, work_bytes, opts, stream);
}

tsqr_status tsqr_float(int m, int n, float* A, int lda, float* R, int ldr, float* d_work, int ldwork) {
    return ref_form<float, false>(m, n, A, lda, R, ldr, d_work, ldwork);
}
tsqr_status tsqr_double(int m, int n, double* A, int lda, double* R, int ldr, double* d_work, int ldwork) {
    return ref_form<double, false>(m, n, A, lda, R, ldr, d_work, ldwork);
}
tsqr_status qr_float(int m, int n, float* A, int lda, float* R, int ldr, float* d_work, int ldwork) {
    return ref_form<float, true>(m, n, A, lda, R, ldr, d_work, ldwork);
}
tsqr_status qr_double(int m, int n, double* A, int lda, double* R, int ldr, double* d_work, int ldwork) {
    return ref_form<double, true>(m, n, A, lda, R, ldr, d_work, ldwork);
}

size_t tsqr_batched_workspace_bytes(int count, const int64_t* m, const int64_t* n) {
    if (count < 0 || (count > 0 && (m == nullptr || n == nullptr))) return 0;
    return tsqr::batched_workspace(count, m, n);
}

tsqr_status tsqr_batched_tune_s(int count, const int64_t* m, const int64_t* n, int reps, void* stream) {
    return tsqr::batched_tune(count, m, n, reps, (cudaStream_t)stream);
}
int tsqr_batched_choice(int width_class, int height_bucket) {
    return tsqr::batched_choice(width_class, height_bucket);
}
int tsqr_batched_candidate_rows(int width_class, int candidate) {
    return tsqr::batched_candidate_rows(width_class, candidate);
}
tsqr_status tsqr_batched_set_choice(int width_class, int height_bucket, int candidate) {
    return tsqr::batched_set_choice(width_class, height_bucket, candidate);
}

tsqr_status tsqr_batched_s(int count, float* const* A, const int64_t* m, const int64_t* n, const int64_t* lda,
                           float* const* R, const int64_t* ldr, void* work, size_t work_bytes,
                           const tsqr_opts* opts, void* stream) {
    const tsqr_opts o = opts_or_default(opts);
    if (count < 0) return TSQR_ERR_INVALID_ARG;
    if (count == 0) return TSQR_OK;
    if (!A || !m || !n || !lda || !R || !ldr) return TSQR_ERR_INVALID_ARG;
    for (int i = 0; i < 2; ++i)
        if (o.reserved[i] != 0) return TSQR_ERR_INVALID_ARG;
    if (o.algorithm != TSQR_QR_BLOCK_GS && o.algorithm != TSQR_QR_HOUSEHOLDER) return TSQR_ERR_INVALID_ARG;
    if (o.precision != TSQR_PRECISION_PLAIN || o.fp64_scalars || o.fp64_root) return TSQR_ERR_UNSUPPORTED;
    for (int i = 0; i < count; ++i) {
        if (m[i] < 1 || n[i] < 1 || m[i] < n[i] || lda[i] < m[i] || ldr[i] < n[i]) return TSQR_ERR_INVALID_ARG;
        if (A[i] == nullptr || R[i] == nullptr) return TSQR_ERR_INVALID_ARG;
        if (n[i] > 64 || m[i] > INT32_MAX) return TSQR_ERR_UNSUPPORTED;
    }
    return tsqr::batched_run(count, A, m, n, lda, R, ldr, work, work_bytes, (cudaStream_t)stream);
}

const char* tsqr_status_string(tsqr_status s) {
    switch (s) {
        case TSQR_OK: return "success";
        case TSQR_ERR_INVALID_ARG: return "invalid argument (m, n, lda, ldr, pointer or options)";
        case TSQR_ERR_UNSUPPORTED: return "size or option not supported";
        case TSQR_ERR_WORKSPACE: return "workspace missing or too small";
        case TSQR_ERR_CUDA: return "CUDA runtime error";
        case TSQR_ERR_NO_DEVICE: return "no usable CUDA device";
    }
    return "unknown status";
}

const char* tsqr_version(void) { return "0.1.0"; }

tsqr_status tsqr_debug_set_wait_limit(int polls) {
    tsqr::wait_tries().store(polls < 0 ? tsqr::kDefaultWaitTries : polls, std::memory_order_relaxed);
    return TSQR_OK;
}

tsqr_status tsqr_profile(int kind, int elem_bytes, int64_t m, int64_t n, void* A, int64_t lda, void* R, int64_t ldr,
                         void* work, size_t work_bytes, const tsqr_opts* opts, void* stream, float* launch_ms,
                         int* launch_tag, int max_launch, int* n_launch) {
    if (!launch_ms || !launch_tag || !n_launch || max_launch < 1) return TSQR_ERR_INVALID_ARG;
    if (kind < 0 || kind > 1 || (elem_bytes != 4 && elem_bytes != 8)) return TSQR_ERR_INVALID_ARG;
    tsqr::LaunchLog* log = new tsqr::LaunchLog();
    const int nev = tsqr::LaunchLog::kMax + 1;
    for (int i = 0; i < nev; ++i) cudaEventCreate(&log->ev[i]);
    cudaStream_t s = (cudaStream_t)stream;
    cudaEventRecord(log->ev[0], s);
    tsqr::tl_log = log;
    tsqr_status st;
    if (kind == 0)
        st = elem_bytes == 4 ? tsqr_s_ex(m, n, (float*)A, lda, (float*)R, ldr, work, work_bytes, opts, stream)
                             : tsqr_d_ex(m, n, (double*)A, lda, (double*)R, ldr, work, work_bytes, opts, stream);
    else
        st = elem_bytes == 4 ? qr_s_ex(m, n, (float*)A, lda, (float*)R, ldr, work, work_bytes, opts, stream)
                             : qr_d_ex(m, n, (double*)A, lda, (double*)R, ldr, work, work_bytes, opts, stream);
    tsqr::tl_log = nullptr;
    int cnt = log->count;
    if (st == TSQR_OK && cudaEventSynchronize(log->ev[cnt]) != cudaSuccess) st = TSQR_ERR_CUDA;
    *n_launch = 0;
    if (st == TSQR_OK) {
        int k = cnt < max_launch ? cnt : max_launch;
        for (int i = 0; i < k; ++i) {
            float ms = 0;
            cudaEventElapsedTime(&ms, log->ev[i], log->ev[i + 1]);
            launch_ms[i] = ms;
            launch_tag[i] = log->tag[i];
        }
        *n_launch = k;
    }
    for (int i = 0; i < nev; ++i) cudaEventDestroy(log->ev[i]);
    delete log;
    return st;
}

}  // extern "C"
