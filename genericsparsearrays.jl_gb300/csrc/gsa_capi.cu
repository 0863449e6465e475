// extern "C" entry points of libgsa (declared in include/gsa.h): argument and
// dimension checks in the order the reference's mul! methods make them,
// dispatch to the kernels, stream-ordered workspace, error strings.
#include <new>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "gsa_internal.cuh"

namespace gsa {

static thread_local char g_err[512] = "";
static thread_local cudaEvent_t g_timer_before = nullptr, g_timer_after = nullptr;

void timer_before(cudaStream_t s) {
    if (g_timer_before) cudaEventRecord(g_timer_before, s);
}
void timer_after(cudaStream_t s) {
    if (g_timer_after) cudaEventRecord(g_timer_after, s);
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return status;
}

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return GSA_OK;
    return fail(GSA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Workspace: the caller's, or a stream-ordered allocation released on the
// same stream once the enqueued work is done with it.

static bool misaligned(const void *p, size_t a) { return a && ((uintptr_t)p % a) != 0; }

// Shared checks of the mul! entry points: sizes of op(A), op(B), C.
static int check_mul_args(int dtype, int itype, int64_t m, int64_t n, int64_t nnz, int opA,
                          int64_t k, int64_t ldb, int opB, int64_t ldc, const void *alpha,
                          const void *beta, const void *B, const void *C, const void *const *arrs,
                          int narr) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (opA < 0 || opA > 2 || opB < 0 || opB > 2)
        return fail(GSA_ERR_INVALID_ARG, "op must be 0 (N), 1 (T) or 2 (C)");
    if (m < 0 || n < 0 || nnz < 0 || k < 0)
        return fail(GSA_ERR_INVALID_ARG, "negative size (m=%lld n=%lld nnz=%lld k=%lld)",
                    (long long)m, (long long)n, (long long)nnz, (long long)k);
    if (!alpha || !beta) return fail(GSA_ERR_INVALID_ARG, "alpha and beta must be host pointers");
    if (itype == GSA_IDX32 && nnz > 0x7fffffffLL)  // Int32 pointers cannot address more
        return fail(GSA_ERR_INVALID_ARG, "nnz=%lld exceeds what Int32 indices can address", (long long)nnz);
    int64_t rows_out = opA == GSA_OP_N ? m : n;
    int64_t inner = opA == GSA_OP_N ? n : m;
    int64_t need_ldb = opB == GSA_OP_N ? inner : k;
    if (ldb < (need_ldb > 1 ? need_ldb : 1))
        return fail(GSA_ERR_DIM, "ldb=%lld is smaller than %lld", (long long)ldb, (long long)need_ldb);
    if (ldc < (rows_out > 1 ? rows_out : 1))
        return fail(GSA_ERR_DIM, "ldc=%lld is smaller than %lld", (long long)ldc, (long long)rows_out);
    if (rows_out > 0 && k > 0 && !C) return fail(GSA_ERR_INVALID_ARG, "C is NULL");
    if (inner > 0 && k > 0 && !B) return fail(GSA_ERR_INVALID_ARG, "B is NULL");
    if (misaligned(B, vs) || misaligned(C, vs))
        return fail(GSA_ERR_INVALID_ARG, "dense operands must be aligned to their element size");
    for (int i = 0; i < narr; ++i) {
        size_t a = (i == narr - 1) ? vs : is;
        if (misaligned(arrs[i], a))
            return fail(GSA_ERR_INVALID_ARG, "sparse arrays must be aligned to their element size");
    }
    return GSA_OK;
}

template <typename V> static DenseIn<V> make_in(const void *B, int64_t ldb, int opB) {
    DenseIn<V> d;
    d.p = (const V *)B;
    d.rs = opB == GSA_OP_N ? 1 : ldb;
    d.cs = opB == GSA_OP_N ? ldb : 1;
    d.conj = opB == GSA_OP_C;
    return d;
}

template <typename V>
static DenseOut<V> make_out(void *C, int64_t ldc, const void *alpha, const void *beta) {
    DenseOut<V> d;
    d.p = (V *)C;
    d.ld = ldc;
    memcpy(&d.alpha, alpha, sizeof(V));
    memcpy(&d.beta, beta, sizeof(V));
    d.beta_mode = beta_mode_of(d.beta);
    d.alpha_one = alpha_one_of(d.alpha);
    return d;
}

struct CompressedMulBody {
    cudaStream_t s; bool gather; int64_t outer_n, inner_n, nnz, k, rows_out;
    const void *ptr, *idx, *val, *B, *alpha, *beta; void *C; int base, opA, opB, algo;
    int64_t ldb, ldc; void *ws; size_t ws_bytes; const Plan *plan;
    template <typename V, typename I> int operator()() {
        CompressedArgs<V, I> a;
        a.outer_n = outer_n; a.inner_n = inner_n; a.nnz = nnz;
        a.ptr = (const I *)ptr; a.idx = (const I *)idx; a.val = (const V *)val;
        a.base = base; a.conjA = (opA == GSA_OP_C);
        DenseIn<V> Bv = make_in<V>(B, ldb, opB);
        DenseOut<V> Cv = make_out<V>(C, ldc, alpha, beta);
        if (rows_out == 0 || k == 0) return GSA_OK;
        Workspace w;
        size_t need = gather ? gather_workspace_size<V, I>(outer_n, nnz, k, algo, plan)
                             : scatter_workspace_size<V, I>(outer_n, nnz, k, algo);
        int rc = w.acquire(s, ws, ws_bytes, need);
        if (rc) return rc;
        if (gather) return launch_gather<V, I>(s, a, k, Bv, Cv, algo, plan, w.p, w.bytes);
        return launch_scatter<V, I>(s, a, k, Bv, Cv, rows_out, algo, plan, w.p, w.bytes);
    }
};

struct CooMulBody {
    cudaStream_t s; bool trans; int64_t nnz, k, rows_out, in_rows;
    const void *rowind, *colind, *val, *B, *alpha, *beta; void *C; int base, opA, opB;
    int64_t ldb, ldc;
    template <typename V, typename I> int operator()() {
        DenseIn<V> Bv = make_in<V>(B, ldb, opB);
        DenseOut<V> Cv = make_out<V>(C, ldc, alpha, beta);
        if (rows_out == 0 || k == 0) return GSA_OK;
        const I *out_idx = (const I *)(trans ? colind : rowind);
        const I *in_idx = (const I *)(trans ? rowind : colind);
        return launch_coo<V, I>(s, nnz, out_idx, in_idx, (const V *)val, base, opA == GSA_OP_C, k,
                                Bv, Cv, rows_out, in_rows);
    }
};

struct MulWsBody {
    bool gather; int64_t outer_n, nnz, k; int algo; size_t out; const Plan *plan;
    template <typename V, typename I> int operator()() {
        out = gather ? gather_workspace_size<V, I>(outer_n, nnz, k, algo, plan)
                     : scatter_workspace_size<V, I>(outer_n, nnz, k, algo);
        return 0;
    }
};

struct CooToCompressedBody {
    cudaStream_t s; bool colmajor; int64_t m, n, nnz; const void *r, *c, *v; int base;
    void *po, *io, *vo, *ws; size_t ws_bytes;
    template <typename V, typename I> int operator()() {
        Workspace w;
        int rc = w.acquire(s, ws, ws_bytes, coo_to_compressed_workspace_size<V, I>(m, n, nnz, colmajor));
        if (rc) return rc;
        return launch_coo_to_compressed<V, I>(s, colmajor, m, n, nnz, (const I *)r, (const I *)c,
                                              (const V *)v, base, (I *)po, (I *)io, (V *)vo, w.p,
                                              w.bytes);
    }
};

struct NoallocSpmvBody {
    cudaStream_t s; int64_t m, n, nnz; const void *ptr, *idx, *val, *x, *alpha, *beta; void *y;
    int base;
    template <typename V, typename I> int operator()() {
        CompressedArgs<V, I> a;
        a.outer_n = m; a.inner_n = n; a.nnz = nnz;
        a.ptr = (const I *)ptr; a.idx = (const I *)idx; a.val = (const V *)val;
        a.base = base; a.conjA = false;
        DenseIn<V> Bv = make_in<V>(x, n > 1 ? n : 1, GSA_OP_N);
        DenseOut<V> Cv = make_out<V>(y, m > 1 ? m : 1, alpha, beta);
        return launch_spmv_noalloc<V, I>(s, a, Bv, Cv);
    }
};

struct CooToCompressedWsBody {
    bool colmajor; int64_t m, n, nnz; size_t out;
    template <typename V, typename I> int operator()() {
        out = coo_to_compressed_workspace_size<V, I>(m, n, nnz, colmajor);
        return 0;
    }
};

// CSR and CSC share one body: 'compressed rows' decides whether opA == N is a
// gather (CSR) or a scatter (CSC).
static int compressed_mul(bool csr, void *stream, int dtype, int itype, int64_t m, int64_t n,
                          int64_t nnz, const void *ptr, const void *idx, const void *val, int base,
                          int opA, int64_t k, const void *B, int64_t ldb, int opB, void *C,
                          int64_t ldc, const void *alpha, const void *beta, int algo, void *ws,
                          size_t ws_bytes, const Plan *plan = nullptr) {
    const void *arrs[3] = {ptr, idx, val};
    int rc = check_mul_args(dtype, itype, m, n, nnz, opA, k, ldb, opB, ldc, alpha, beta, B, C, arrs, 3);
    if (rc) return rc;
    if (!ptr) return fail(GSA_ERR_INVALID_ARG, "pointer array is NULL");
    if (nnz > 0 && (!idx || !val)) return fail(GSA_ERR_INVALID_ARG, "index/value arrays are NULL");
    if (algo < 0 || algo > 3) return fail(GSA_ERR_INVALID_ARG, "unknown algo %d", algo);
    if (plan && (plan->outer_n != (csr ? m : n) || plan->nnz != nnz))
        return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
    cudaStream_t s = (cudaStream_t)stream;
    const bool gather = csr ? (opA == GSA_OP_N) : (opA != GSA_OP_N);
    const int64_t outer_n = csr ? m : n, inner_n = csr ? n : m;
    const int64_t rows_out = opA == GSA_OP_N ? m : n;
    CompressedMulBody body{s, gather, outer_n, inner_n, nnz, k, rows_out, ptr, idx, val, B, alpha,
                           beta, C, base, opA, opB, algo, ldb, ldc, ws, ws_bytes, plan};
    return dispatch_vi(dtype, itype, body);
}

}  // namespace gsa

using namespace gsa;

extern "C" {

int gsa_version(void) { return 100; }

const char *gsa_last_error_string(void) { return g_err; }

void gsa_set_kernel_timer(void *before, void *after) {
    g_timer_before = (cudaEvent_t)before;
    g_timer_after = (cudaEvent_t)after;
}

int gsa_csr_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowptr, const void *colval, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta, int algo, void *workspace,
                size_t workspace_bytes) {
    return compressed_mul(true, stream, dtype, itype, m, n, nnz, rowptr, colval, nzval, base, opA,
                          k, B, ldb, opB, C, ldc, alpha, beta, algo, workspace, workspace_bytes);
}

int gsa_csc_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *colptr, const void *rowval, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta, int algo, void *workspace,
                size_t workspace_bytes) {
    return compressed_mul(false, stream, dtype, itype, m, n, nnz, colptr, rowval, nzval, base, opA,
                          k, B, ldb, opB, C, ldc, alpha, beta, algo, workspace, workspace_bytes);
}

int gsa_plan_create(void *stream, int itype, int64_t outer_n, int64_t nnz, const void *ptr, int base,
                    gsa_plan **out) {
    if (!out) return fail(GSA_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!itype_size(itype)) return fail(GSA_ERR_UNSUPPORTED, "unsupported itype %d", itype);
    if (outer_n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (!ptr) return fail(GSA_ERR_INVALID_ARG, "pointer array is NULL");
    Plan *p = new (std::nothrow) Plan();
    if (!p) return fail(GSA_ERR_ALLOC, "plan: host memory");
    int rc = plan_create((cudaStream_t)stream, itype, outer_n, nnz, ptr, base, p);
    if (rc) {
        if (p->mem) cudaFree(p->mem);
        delete p;
        return rc;
    }
    *out = p;
    return GSA_OK;
}

int gsa_coo_plan_create(void *stream, int itype, int64_t m, int64_t n, int64_t nnz, const void *rowind,
                        int base, gsa_plan **out) {
    if (!out) return fail(GSA_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    const size_t is = itype_size(itype);
    if (!is) return fail(GSA_ERR_UNSUPPORTED, "unsupported itype %d", itype);
    if (m < 0 || n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (nnz > 0 && !rowind) return fail(GSA_ERR_INVALID_ARG, "rowind is NULL");
    if (misaligned(rowind, is)) return fail(GSA_ERR_INVALID_ARG, "rowind must be aligned to its element size");
    if (itype == GSA_IDX32 && nnz > 0x7fffffffLL)
        return fail(GSA_ERR_INVALID_ARG, "nnz=%lld exceeds what Int32 indices can address", (long long)nnz);
    Plan *p = new (std::nothrow) Plan();
    if (!p) return fail(GSA_ERR_ALLOC, "plan: host memory");
    p->coo = 1;
    p->outer_n = m;
    p->nnz = nnz;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = check_cuda(cudaMalloc(&p->coo_ptr, is * (size_t)(m + 1)), "coo plan: row pointers");
    int sorted = 0;
    if (!rc) rc = coo_row_pointers(s, itype, m, nnz, rowind, base, p->coo_ptr, &sorted);
    if (!rc && sorted) {
        p->coo_sorted = 1;
        rc = plan_create(s, itype, m, nnz, p->coo_ptr, base, p);
    }
    if (!rc && !sorted) {  // the COO kernel keeps it; drop the pointers
        cudaFree(p->coo_ptr);
        p->coo_ptr = nullptr;
    }
    if (rc) {
        if (p->mem) cudaFree(p->mem);
        if (p->coo_ptr) cudaFree(p->coo_ptr);
        delete p;
        return rc;
    }
    *out = p;
    return GSA_OK;
}

int gsa_plan_bin_order(const gsa_plan *plan, const void **view, int64_t *warps) {
    if (!plan || !view || !warps) return fail(GSA_ERR_INVALID_ARG, "NULL argument");
    // grouped launches take the bin order only without rows of more than one chunk (those
    // need a call's partial sums)
    const bool ok = plan->nbin_warps > 0 && plan->bin_view && plan->bin.nlong == 0;
    *view = ok ? (const void *)plan->bin_view : nullptr;
    *warps = ok ? plan->nbin_warps : 0;
    return GSA_OK;
}

int gsa_coo_plan_info(const gsa_plan *plan, int *row_sorted) {
    if (!plan || !row_sorted) return fail(GSA_ERR_INVALID_ARG, "NULL argument");
    *row_sorted = plan->coo ? plan->coo_sorted : 0;
    return GSA_OK;
}

int gsa_coo_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *rowind, const void *colind, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes) {
    if (plan && !plan->coo) return fail(GSA_ERR_INVALID_ARG, "not a COO plan");
    if (plan && (plan->outer_n != m || plan->nnz != nnz))
        return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
    if (!plan || !plan->coo_sorted)
        return gsa_coo_mul(stream, dtype, itype, m, n, nnz, rowind, colind, nzval, base, opA, k, B, ldb,
                           opB, C, ldc, alpha, beta);
    // row-sorted: the CSR kernels on (plan row pointers, colind, nzval)
    return compressed_mul(true, stream, dtype, itype, m, n, nnz, plan->coo_ptr, colind, nzval, base, opA,
                          k, B, ldb, opB, C, ldc, alpha, beta, GSA_ALGO_AUTO, workspace, workspace_bytes,
                          plan);
}

int gsa_plan_destroy(gsa_plan *plan) {
    if (!plan) return GSA_OK;
    int rc = GSA_OK;
    if (plan->coo_ptr) cudaFree(plan->coo_ptr);
    if (plan->mem) rc = check_cuda(cudaFree(plan->mem), "plan: free");
    delete plan;
    return rc;
}

int gsa_plan_info(const gsa_plan *plan, int64_t *max_len, int64_t *nlong, int64_t *nchunks) {
    if (!plan) return fail(GSA_ERR_INVALID_ARG, "plan is NULL");
    if (max_len) *max_len = plan->max_len;
    if (nlong) *nlong = plan->nplanned;
    if (nchunks) *nchunks = plan->nbin_warps > 0 ? plan->bin.nchunks : plan->nat.nchunks;
    return GSA_OK;
}

int gsa_csr_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *rowptr, const void *colval, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes) {
    return compressed_mul(true, stream, dtype, itype, m, n, nnz, rowptr, colval, nzval, base, opA,
                          k, B, ldb, opB, C, ldc, alpha, beta, GSA_ALGO_AUTO, workspace,
                          workspace_bytes, plan);
}

int gsa_csc_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *colptr, const void *rowval, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes) {
    return compressed_mul(false, stream, dtype, itype, m, n, nnz, colptr, rowval, nzval, base, opA,
                          k, B, ldb, opB, C, ldc, alpha, beta, GSA_ALGO_AUTO, workspace,
                          workspace_bytes, plan);
}

size_t gsa_plan_workspace_size(const gsa_plan *plan, int dtype, int64_t k) {
    return rowblock_workspace_size(plan, dtype_size(dtype), k);
}

int gsa_coo_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowind, const void *colind, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta) {
    const void *arrs[3] = {rowind, colind, nzval};
    int rc = check_mul_args(dtype, itype, m, n, nnz, opA, k, ldb, opB, ldc, alpha, beta, B, C, arrs, 3);
    if (rc) return rc;
    if (nnz > 0 && (!rowind || !colind || !nzval))
        return fail(GSA_ERR_INVALID_ARG, "COO arrays are NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const bool trans = opA != GSA_OP_N;
    const int64_t rows_out = trans ? n : m, in_rows = trans ? m : n;
    CooMulBody body{s, trans, nnz, k, rows_out, in_rows, rowind, colind, nzval, B, alpha, beta, C,
                    base, opA, opB, ldb, ldc};
    return dispatch_vi(dtype, itype, body);
}

}  // extern "C"

namespace gsa {
struct DotBody {
    cudaStream_t s; int fmt, opA; int64_t m, n, nnz; const void *p0, *p1, *val, *x, *y; int base;
    const Plan *plan; void *ws; size_t ws_bytes; void *result;
    template <typename V, typename I> int operator()() {
        Workspace w;
        int rc = w.acquire(s, ws, ws_bytes, dot_workspace_size<V, I>(fmt, fmt == 0 ? m : n, plan));
        if (rc) return rc;
        return launch_dot<V, I>(s, fmt, opA, m, n, nnz, (const I *)p0, (const I *)p1, (const V *)val, base,
                                (const V *)x, (const V *)y, plan, w.p, w.bytes, result);
    }
};
struct DotWsBody {
    int fmt; int64_t outer_n; const Plan *plan; size_t out;
    template <typename V, typename I> int operator()() {
        out = dot_workspace_size<V, I>(fmt, outer_n, plan);
        return 0;
    }
};

static int dot_call(int fmt, void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                    const void *p0, const void *p1, const void *val, int base, int opA, const void *x,
                    const void *y, void *result, const gsa_plan *plan, void *ws, size_t ws_bytes) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (opA < 0 || opA > 2) return fail(GSA_ERR_INVALID_ARG, "op must be 0 (N), 1 (T) or 2 (C)");
    if (m < 0 || n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (itype == GSA_IDX32 && nnz > 0x7fffffffLL)
        return fail(GSA_ERR_INVALID_ARG, "nnz=%lld exceeds what Int32 indices can address", (long long)nnz);
    if (!result) return fail(GSA_ERR_INVALID_ARG, "result must be a host pointer");
    const int64_t xlen = opA == GSA_OP_N ? m : n, ylen = opA == GSA_OP_N ? n : m;
    if ((xlen > 0 && !x) || (ylen > 0 && !y)) return fail(GSA_ERR_INVALID_ARG, "x or y is NULL");
    if (fmt != 2 && !p0) return fail(GSA_ERR_INVALID_ARG, "pointer array is NULL");
    if (nnz > 0 && (!p0 || !p1 || !val)) return fail(GSA_ERR_INVALID_ARG, "sparse arrays are NULL");
    if (misaligned(p0, is) || misaligned(p1, is) || misaligned(val, vs) || misaligned(x, vs) ||
        misaligned(y, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    if (plan && fmt != 2 && (plan->outer_n != (fmt == 0 ? m : n) || plan->nnz != nnz))
        return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
    DotBody body{(cudaStream_t)stream, fmt, opA, m, n, nnz, p0, p1, val, x, y, base,
                 fmt == 2 ? nullptr : plan, ws, ws_bytes, result};
    return dispatch_vi(dtype, itype, body);
}
}  // namespace gsa

extern "C" {

int gsa_csr_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz, const void *rowptr,
                const void *colval, const void *nzval, int base, int opA, const void *x, const void *y,
                void *result, const gsa_plan *plan, void *workspace, size_t workspace_bytes) {
    return dot_call(0, stream, dtype, itype, m, n, nnz, rowptr, colval, nzval, base, opA, x, y, result,
                    plan, workspace, workspace_bytes);
}

int gsa_csc_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz, const void *colptr,
                const void *rowval, const void *nzval, int base, int opA, const void *x, const void *y,
                void *result, const gsa_plan *plan, void *workspace, size_t workspace_bytes) {
    return dot_call(1, stream, dtype, itype, m, n, nnz, colptr, rowval, nzval, base, opA, x, y, result,
                    plan, workspace, workspace_bytes);
}

int gsa_coo_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz, const void *rowind,
                const void *colind, const void *nzval, int base, int opA, const void *x, const void *y,
                void *result, const gsa_plan *plan, void *workspace, size_t workspace_bytes) {
    if (plan && (!plan->coo || plan->outer_n != m || plan->nnz != nnz))
        return fail(GSA_ERR_INVALID_ARG, "plan is not a COO plan of this structure");
    if (plan && plan->coo_sorted)  // row-sorted: the CSR dot on the plan's row pointers
        return dot_call(0, stream, dtype, itype, m, n, nnz, plan->coo_ptr, colind, nzval, base, opA, x, y,
                        result, plan, workspace, workspace_bytes);
    return dot_call(2, stream, dtype, itype, m, n, nnz, rowind, colind, nzval, base, opA, x, y, result,
                    nullptr, workspace, workspace_bytes);
}

}  // extern "C"

namespace gsa {
struct DropCountBody {
    cudaStream_t s; int64_t nnz; const void *val; void *ws; size_t ws_bytes; int64_t *kept;
    template <typename V, typename I> int operator()() {
        return launch_dropzeros_count<V>(s, nnz, (const V *)val, ws, ws_bytes, kept);
    }
};
struct DropCopyBody {
    cudaStream_t s; int fmt; int64_t outer_n, nnz; const void *p0, *p1, *val; int base; const void *ws;
    void *o0, *o1, *ov;
    template <typename V, typename I> int operator()() {
        return launch_dropzeros_copy<V, I>(s, fmt, outer_n, nnz, (const I *)p0, (const I *)p1, (const V *)val,
                                           base, ws, (I *)o0, (I *)o1, (V *)ov);
    }
};
struct SumCountBody {
    cudaStream_t s; int64_t m, n; SumSources src; const void *lambda; int base; void *ws; size_t ws_bytes;
    int64_t *kept;
    template <typename V, typename I> int operator()() {
        return launch_coo_sum_count<V, I>(s, m, n, src, (const V *)lambda, base, ws, ws_bytes, kept);
    }
};
struct SumCopyBody {
    cudaStream_t s; int64_t m, n, total; int base; const void *ws; void *ro, *co, *vo;
    template <typename V, typename I> int operator()() {
        return launch_coo_sum_copy<V, I>(s, m, n, total, base, ws, (I *)ro, (I *)co, (V *)vo);
    }
};
struct AddBody {
    cudaStream_t s; int fmt; int64_t m, n, nnz; const void *p0, *p1, *val; int base; void *C; int64_t ldc;
    template <typename V, typename I> int operator()() {
        return launch_add_to_dense<V, I>(s, fmt, m, n, nnz, (const I *)p0, (const I *)p1, (const V *)val, base,
                                         (V *)C, ldc);
    }
};
}  // namespace gsa

extern "C" {

size_t gsa_dropzeros_workspace_size(int64_t nnz) { return nnz < 0 ? 0 : dropzeros_workspace_size(nnz); }

int gsa_dropzeros_count(void *stream, int dtype, int64_t nnz, const void *nzval, void *workspace,
                        size_t workspace_bytes, int64_t *kept) {
    const size_t vs = dtype_size(dtype);
    if (!vs) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d", dtype);
    if (nnz < 0 || !kept || !workspace) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (nnz > 0 && !nzval) return fail(GSA_ERR_INVALID_ARG, "nzval is NULL");
    if (misaligned(nzval, vs)) return fail(GSA_ERR_INVALID_ARG, "nzval must be aligned to its element size");
    DropCountBody body{(cudaStream_t)stream, nnz, nzval, workspace, workspace_bytes, kept};
    return dispatch_vi(dtype, GSA_IDX64, body);
}

int gsa_dropzeros_copy(void *stream, int format, int dtype, int itype, int64_t outer_n, int64_t nnz,
                       const void *p0, const void *p1, const void *nzval, int base, const void *workspace,
                       void *p0_out, void *p1_out, void *val_out) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (format < 0 || format > 2) return fail(GSA_ERR_INVALID_ARG, "format must be 0 (CSR), 1 (CSC) or 2 (COO)");
    if (outer_n < 0 || nnz < 0 || !workspace) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (format != 2 && (!p0 || !p0_out)) return fail(GSA_ERR_INVALID_ARG, "pointer arrays are NULL");
    if (nnz > 0 && (!p1 || !nzval || (format == 2 && !p0))) return fail(GSA_ERR_INVALID_ARG, "sparse arrays are NULL");
    if (misaligned(p0, is) || misaligned(p1, is) || misaligned(nzval, vs) || misaligned(p0_out, is) ||
        misaligned(p1_out, is) || misaligned(val_out, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    DropCopyBody body{(cudaStream_t)stream, format, outer_n, nnz, p0, p1, nzval, base, workspace, p0_out, p1_out,
                      val_out};
    return dispatch_vi(dtype, itype, body);
}

size_t gsa_coo_sum_workspace_size(int dtype, int64_t m, int64_t n, int64_t total) {
    const size_t vs = dtype_size(dtype);
    return !vs || total < 0 || m < 0 || n < 0 ? 0 : coo_sum_workspace_size(vs, m, n, total);
}

int gsa_coo_sum_count(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz_a,
                      const void *rowind_a, const void *colind_a, const void *nzval_a, int op_a, int64_t nnz_b,
                      const void *rowind_b, const void *colind_b, const void *nzval_b, int op_b, int64_t n_diag,
                      const void *lambda, int base, void *workspace, size_t workspace_bytes, int64_t *kept) {
    const size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (m < 0 || n < 0 || nnz_a < 0 || nnz_b < 0 || n_diag < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (!kept || !workspace) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    const int ops[2] = {op_a, op_b};
    for (int w = 0; w < 2; ++w)
        if ((ops[w] & ~GSA_SUM_NEGATE) < GSA_OP_N || (ops[w] & ~GSA_SUM_NEGATE) > GSA_OP_C)
            return fail(GSA_ERR_INVALID_ARG, "op_%c must be GSA_OP_N, T or C, optionally | GSA_SUM_NEGATE",
                        w ? 'b' : 'a');
    if (n_diag > (m < n ? m : n)) return fail(GSA_ERR_DIM, "n_diag=%lld exceeds min(m, n)", (long long)n_diag);
    if (n_diag > 0 && !lambda) return fail(GSA_ERR_INVALID_ARG, "lambda is NULL");
    if ((nnz_a > 0 && (!rowind_a || !colind_a || !nzval_a)) || (nnz_b > 0 && (!rowind_b || !colind_b || !nzval_b)))
        return fail(GSA_ERR_INVALID_ARG, "sparse arrays are NULL");
    if (misaligned(rowind_a, is) || misaligned(colind_a, is) || misaligned(nzval_a, vs) || misaligned(rowind_b, is) ||
        misaligned(colind_b, is) || misaligned(nzval_b, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    SumSources src{};
    src.row[0] = rowind_a; src.col[0] = colind_a; src.val[0] = nzval_a; src.nnz[0] = nnz_a;
    src.row[1] = rowind_b; src.col[1] = colind_b; src.val[1] = nzval_b; src.nnz[1] = nnz_b;
    src.n_diag = n_diag;
    for (int w = 0; w < 2; ++w) {
        const int op = ops[w] & ~GSA_SUM_NEGATE;
        src.trans[w] = op != GSA_OP_N;
        src.conj[w] = op == GSA_OP_C;
        src.neg[w] = (ops[w] & GSA_SUM_NEGATE) != 0;
    }
    SumCountBody body{(cudaStream_t)stream, m, n, src, lambda, base, workspace, workspace_bytes, kept};
    return dispatch_vi(dtype, itype, body);
}

int gsa_coo_sum_copy(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t total, int64_t kept,
                     int base, const void *workspace, void *rowind_out, void *colind_out, void *nzval_out) {
    const size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (m < 0 || n < 0 || total < 0 || kept < 0 || kept > total || !workspace)
        return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (kept == 0) return GSA_OK;
    if (!rowind_out || !colind_out || !nzval_out) return fail(GSA_ERR_INVALID_ARG, "outputs are NULL");
    if (misaligned(rowind_out, is) || misaligned(colind_out, is) || misaligned(nzval_out, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    SumCopyBody body{(cudaStream_t)stream, m, n, total, base, workspace, rowind_out, colind_out, nzval_out};
    return dispatch_vi(dtype, itype, body);
}

int gsa_add_to_dense(void *stream, int format, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                     const void *p0, const void *p1, const void *nzval, int base, void *C, int64_t ldc) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (format < 0 || format > 2) return fail(GSA_ERR_INVALID_ARG, "format must be 0 (CSR), 1 (CSC) or 2 (COO)");
    if (m < 0 || n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (itype == GSA_IDX32 && nnz > 0x7fffffffLL)
        return fail(GSA_ERR_INVALID_ARG, "nnz=%lld exceeds what Int32 indices can address", (long long)nnz);
    if (ldc < (m > 1 ? m : 1)) return fail(GSA_ERR_DIM, "ldc=%lld is smaller than %lld", (long long)ldc, (long long)m);
    if (m > 0 && n > 0 && !C) return fail(GSA_ERR_INVALID_ARG, "C is NULL");
    if (format != 2 && !p0) return fail(GSA_ERR_INVALID_ARG, "pointer array is NULL");
    if (nnz > 0 && (!p0 || !p1 || !nzval)) return fail(GSA_ERR_INVALID_ARG, "sparse arrays are NULL");
    if (misaligned(p0, is) || misaligned(p1, is) || misaligned(nzval, vs) || misaligned(C, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    AddBody body{(cudaStream_t)stream, format, m, n, nnz, p0, p1, nzval, base, C, ldc};
    return dispatch_vi(dtype, itype, body);
}

size_t gsa_dot_workspace_size(int format, int dtype, int itype, int64_t m, int64_t n, const gsa_plan *plan) {
    if (format < 0 || format > 2) return 0;
    if (format == 2 && plan && plan->coo_sorted) format = 0;  // served by the CSR dot
    DotWsBody body{format, format == 0 ? m : n, format == 2 ? nullptr : plan, 0};
    if (dispatch_vi(dtype, itype, body)) return 0;
    return body.out;
}

size_t gsa_mul_workspace_size(int format, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                              int opA, int64_t k, int algo) {
    if (format != 0 && format != 1) return 0;
    const bool csr = format == 0;
    const bool gather = csr ? (opA == GSA_OP_N) : (opA != GSA_OP_N);
    const int64_t outer_n = csr ? m : n;
    MulWsBody body{gather, outer_n, nnz, k, algo, 0, nullptr};
    if (dispatch_vi(dtype, itype, body)) return 0;
    return body.out;
}

static int coo_to_compressed(bool colmajor, void *stream, int dtype, int itype, int64_t m, int64_t n,
                             int64_t nnz, const void *rowind, const void *colind, const void *nzval,
                             int base, void *ptr_out, void *idx_out, void *val_out, void *ws,
                             size_t ws_bytes) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (m < 0 || n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (!ptr_out) return fail(GSA_ERR_INVALID_ARG, "pointer output is NULL");
    if (nnz > 0 && (!rowind || !colind || !nzval || !idx_out || !val_out))
        return fail(GSA_ERR_INVALID_ARG, "NULL array");
    if (misaligned(rowind, is) || misaligned(colind, is) || misaligned(ptr_out, is) ||
        misaligned(idx_out, is) || misaligned(nzval, vs) || misaligned(val_out, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    cudaStream_t s = (cudaStream_t)stream;
    CooToCompressedBody body{s, colmajor, m, n, nnz, rowind, colind, nzval, base, ptr_out, idx_out,
                             val_out, ws, ws_bytes};
    return dispatch_vi(dtype, itype, body);
}

int gsa_coo_to_csr(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowind, const void *colind, const void *nzval, int base,
                   void *rowptr_out, void *colval_out, void *nzval_out, void *workspace,
                   size_t workspace_bytes) {
    return coo_to_compressed(false, stream, dtype, itype, m, n, nnz, rowind, colind, nzval, base,
                             rowptr_out, colval_out, nzval_out, workspace, workspace_bytes);
}

int gsa_coo_to_csc(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowind, const void *colind, const void *nzval, int base,
                   void *colptr_out, void *rowval_out, void *nzval_out, void *workspace,
                   size_t workspace_bytes) {
    return coo_to_compressed(true, stream, dtype, itype, m, n, nnz, rowind, colind, nzval, base,
                             colptr_out, rowval_out, nzval_out, workspace, workspace_bytes);
}

size_t gsa_coo_to_compressed_workspace_size(int colmajor, int dtype, int itype, int64_t m, int64_t n,
                                            int64_t nnz) {
    CooToCompressedWsBody body{colmajor != 0, m, n, nnz, 0};
    if (dispatch_vi(dtype, itype, body)) return 0;
    return body.out;
}

static int compressed_to_coo(bool colmajor, void *stream, int dtype, int itype, int64_t m, int64_t n,
                             int64_t nnz, const void *ptr, const void *idx, const void *val, int base,
                             void *rowind_out, void *colind_out, void *val_out) {
    size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (m < 0 || n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (!ptr) return fail(GSA_ERR_INVALID_ARG, "pointer array is NULL");
    if (nnz > 0 && (!idx || !val || !rowind_out || !colind_out || !val_out))
        return fail(GSA_ERR_INVALID_ARG, "NULL array");
    if (misaligned(ptr, is) || misaligned(idx, is) || misaligned(rowind_out, is) ||
        misaligned(colind_out, is) || misaligned(val, vs) || misaligned(val_out, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    if (nnz == 0) return GSA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t outer_n = colmajor ? n : m;
    void *major_out = colmajor ? colind_out : rowind_out;
    void *minor_out = colmajor ? rowind_out : colind_out;
    int rc = check_cuda(cudaMemcpyAsync(minor_out, idx, (size_t)nnz * is, cudaMemcpyDeviceToDevice, s),
                        "index copy");
    if (rc) return rc;
    rc = check_cuda(cudaMemcpyAsync(val_out, val, (size_t)nnz * vs, cudaMemcpyDeviceToDevice, s),
                    "value copy");
    if (rc) return rc;
    Workspace w;
    rc = w.acquire(s, nullptr, 0, expand_major_workspace_size(outer_n, nnz));
    if (rc) return rc;
    if (itype == GSA_IDX32)
        return launch_expand_major<int32_t>(s, outer_n, nnz, (const int32_t *)ptr, base,
                                            (int32_t *)major_out, w.p, w.bytes);
    return launch_expand_major<int64_t>(s, outer_n, nnz, (const int64_t *)ptr, base,
                                        (int64_t *)major_out, w.p, w.bytes);
}

int gsa_csr_to_coo(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowptr, const void *colval, const void *nzval, int base,
                   void *rowind_out, void *colind_out, void *nzval_out) {
    return compressed_to_coo(false, stream, dtype, itype, m, n, nnz, rowptr, colval, nzval, base,
                             rowind_out, colind_out, nzval_out);
}

int gsa_csc_to_coo(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *colptr, const void *rowval, const void *nzval, int base,
                   void *rowind_out, void *colind_out, void *nzval_out) {
    return compressed_to_coo(true, stream, dtype, itype, m, n, nnz, colptr, rowval, nzval, base,
                             rowind_out, colind_out, nzval_out);
}

int gsa_csr_spmv_noalloc(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                         const void *rowptr, const void *colval, const void *nzval, int base,
                         const void *x, void *y, const void *alpha, const void *beta) {
    const void *arrs[3] = {rowptr, colval, nzval};
    int rc = check_mul_args(dtype, itype, m, n, nnz, GSA_OP_N, 1, n > 1 ? n : 1, GSA_OP_N,
                            m > 1 ? m : 1, alpha, beta, x, y, arrs, 3);
    if (rc) return rc;
    if (!rowptr) return fail(GSA_ERR_INVALID_ARG, "rowptr is NULL");
    if (nnz > 0 && (!colval || !nzval)) return fail(GSA_ERR_INVALID_ARG, "colval/nzval are NULL");
    if (m == 0) return GSA_OK;
    NoallocSpmvBody body{(cudaStream_t)stream, m, n, nnz, rowptr, colval, nzval, x, alpha, beta, y, base};
    return dispatch_vi(dtype, itype, body);
}

int gsa_set_tuning(int key, int value) {
    if (key == GSA_TUNE_PIPE_THREADS) {
        if (value != 256 && value != 512) return fail(GSA_ERR_INVALID_ARG, "threads must be 256 or 512");
        set_pipe_threads(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_SPMM_COLUMNS) {
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
            return fail(GSA_ERR_INVALID_ARG, "columns per thread must be 0, 1, 2, 4 or 8");
        set_spmm_columns(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_PLAN_ORDER) {
        if (value < 0 || value > 2) return fail(GSA_ERR_INVALID_ARG, "plan order must be 0, 1 or 2");
        set_plan_natural(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_STAGE_ROWS) {
        if (value < 0 || value > 2) return fail(GSA_ERR_INVALID_ARG, "stage rows must be 0, 1 or 2");
        set_stage_rows(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_X_PAIRS) {
        if (value != 0 && value != 1) return fail(GSA_ERR_INVALID_ARG, "x pairs must be 0 or 1");
        set_x_pairs(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_SORT_STAGED) {
        if (value != 0 && value != 1) return fail(GSA_ERR_INVALID_ARG, "sort staged must be 0 or 1");
        set_sort_staged(value);
        return GSA_OK;
    }
    if (key == GSA_TUNE_WAIT_LIMIT) {
        if (value < 0) return fail(GSA_ERR_INVALID_ARG, "wait limit must be >= 0");
        set_wait_limit(value == 0 ? 0u : (uint32_t)value);
        return GSA_OK;
    }
    return fail(GSA_ERR_INVALID_ARG, "unknown tuning key %d", key);
}

int gsa_get_tuning(int key) {
    if (key == GSA_TUNE_PIPE_THREADS) return get_pipe_threads();
    if (key == GSA_TUNE_SPMM_COLUMNS) return get_spmm_columns();
    if (key == GSA_TUNE_PLAN_ORDER) return get_plan_natural();
    if (key == GSA_TUNE_STAGE_ROWS) return get_stage_rows();
    if (key == GSA_TUNE_X_PAIRS) return get_x_pairs();
    if (key == GSA_TUNE_SORT_STAGED) return get_sort_staged();
    if (key == GSA_TUNE_WAIT_LIMIT) {
        const uint32_t w = get_wait_limit();
        return w > 0x7fffffffu ? 0x7fffffff : (int)w;
    }
    return -1;
}

int gsa_check_device_status(void *stream) {
    int flag = 0;
    int rc = read_pipe_error((cudaStream_t)stream, &flag);
    if (rc) return rc;
    if (flag) return fail(GSA_ERR_TIMEOUT, "a bounded device-side wait gave up (error word %d)", flag);
    return GSA_OK;
}

int gsa_validate_compressed(void *stream, int itype, int64_t outer_n, int64_t inner_n, int64_t nnz,
                            const void *ptr, const void *idx, int base) {
    size_t is = itype_size(itype);
    if (!is) return fail(GSA_ERR_UNSUPPORTED, "unsupported itype %d", itype);
    if (outer_n < 0 || inner_n < 0 || nnz < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    if (!ptr || (nnz > 0 && !idx)) return fail(GSA_ERR_INVALID_ARG, "NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    int *d_flag = nullptr;
    int rc = check_cuda(cudaMallocAsync((void **)&d_flag, sizeof(int), s), "validate flag");
    if (rc) return rc;
    cudaMemsetAsync(d_flag, 0, sizeof(int), s);
    rc = itype == GSA_IDX32
             ? launch_validate<int32_t>(s, outer_n, inner_n, nnz, (const int32_t *)ptr,
                                        (const int32_t *)idx, base, d_flag)
             : launch_validate<int64_t>(s, outer_n, inner_n, nnz, (const int64_t *)ptr,
                                        (const int64_t *)idx, base, d_flag);
    int h_flag = 0;
    if (!rc) rc = check_cuda(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s),
                             "validate readback");
    cudaFreeAsync(d_flag, s);
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "validate sync");
    if (rc) return rc;
    if (h_flag)
        return fail(GSA_ERR_STRUCTURE, "malformed compressed structure (%s%s%s%s)",
                    (h_flag & 1) ? "ptr[0] != base; " : "", (h_flag & 2) ? "ptr[end] != nnz+base; " : "",
                    (h_flag & 4) ? "decreasing ptr; " : "", (h_flag & 8) ? "index out of range" : "");
    return GSA_OK;
}

}  // extern "C"
