/*
 * Type-generic body of the CPU oracle.  TEST INFRASTRUCTURE ONLY: this file is
 * compiled into libgsa_oracle.so, which only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load.  The product path never links it.
 *
 * Included once per (value type, index type) pair by gsa_oracle.c with these
 * macros defined:
 *   V, I          value and index C types
 *   SUFFIX        name suffix of the instantiation
 *   V_ZERO        additive identity
 *   V_ADD(a,b)    a + b in the reference's arithmetic (wrapping for integers)
 *   V_MUL(a,b)    a * b in the reference's arithmetic (Julia's complex formula)
 *   V_CONJ(a)     conj(a)
 *   V_EQ_ONE(a)   a == one(a)
 *   V_IS_ZERO(a)  iszero(a)
 *   V_TO_C(a,re,im) widen to two doubles (error oracle)
 */

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* B(i, c) of op(B) for a column-major parent with leading dimension ldb.
 * opB: 0 = identity, 1 = transpose, 2 = adjoint; the TRANSB/CONJB index
 * swap of src/matrix_csr/matrix_csr_kernels.jl:16-18. */
static inline V FN(getB)(const V *B, int64_t ldb, int opB, int64_t i, int64_t c) {
    V v = (opB == 0) ? B[i + c * ldb] : B[c + i * ldb];
    return (opB == 2) ? V_CONJ(v) : v;
}

/* LinearAlgebra._rmul_or_fill!(C, beta) as called before every kernel
 * (src/matrix_csr/matrix_csr.jl:192): beta == 1 leaves C alone, beta == 0
 * fills zero without reading C, otherwise C .*= beta. */
static void FN(rmul_or_fill)(V *C, int64_t rows, int64_t k, int64_t ldc, V beta) {
    if (V_EQ_ONE(beta) || rows == 0 || k == 0) return;
    for (int64_t c = 0; c < k; ++c)
        for (int64_t r = 0; r < rows; ++r) {
            if (V_IS_ZERO(beta)) C[r + c * ldc] = V_ZERO;
            else C[r + c * ldc] = V_MUL(C[r + c * ldc], beta);
        }
}

/* Gather over the compressed dimension: kernel_spmatmul_csr_N!
 * (src/matrix_csr/matrix_csr_kernels.jl:1-22), identical in shape to
 * kernel_spmatmul_csc_T! (src/matrix_csc/matrix_csc_kernels.jl:24-45).
 * One work item per (c, outer): a serial walk of the outer's range, alpha
 * applied once at the end (C[row,k] += tmp * alpha). */
static void FN(gather)(int64_t outer_n, const I *ptr, const I *idx, const V *val, int base,
                       int conjA, int64_t k, const V *B, int64_t ldb, int opB,
                       V *C, int64_t ldc, V alpha, int nthreads) {
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1) collapse(2)
#endif
    for (int64_t c = 0; c < k; ++c) {
        for (int64_t o = 0; o < outer_n; ++o) {
            V tmp = V_ZERO;
            for (int64_t j = (int64_t)ptr[o] - base; j < (int64_t)ptr[o + 1] - base; ++j) {
                V a = conjA ? V_CONJ(val[j]) : val[j];
                V b = FN(getB)(B, ldb, opB, (int64_t)idx[j] - base, c);
                tmp = V_ADD(tmp, V_MUL(a, b));
            }
            C[o + c * ldc] = V_ADD(C[o + c * ldc], V_MUL(tmp, alpha));
        }
    }
}

/* Scatter over the compressed dimension: kernel_spmatmul_csr_T!
 * (src/matrix_csr/matrix_csr_kernels.jl:24-45) and kernel_spmatmul_csc_N!
 * (src/matrix_csc/matrix_csc_kernels.jl:1-22).  axj = B(outer, c) * alpha,
 * then C[idx_j, c] += a_j * axj for every stored entry.  The reference runs
 * these adds as unordered atomics; the oracle runs them in storage order,
 * which is one of the orders the reference may take. */
static void FN(scatter)(int64_t outer_n, const I *ptr, const I *idx, const V *val, int base,
                        int conjA, int64_t k, const V *B, int64_t ldb, int opB,
                        V *C, int64_t ldc, V alpha) {
    for (int64_t c = 0; c < k; ++c) {
        for (int64_t o = 0; o < outer_n; ++o) {
            V axj = V_MUL(FN(getB)(B, ldb, opB, o, c), alpha);
            for (int64_t j = (int64_t)ptr[o] - base; j < (int64_t)ptr[o + 1] - base; ++j) {
                V a = conjA ? V_CONJ(val[j]) : val[j];
                int64_t r = (int64_t)idx[j] - base;
                C[r + c * ldc] = V_ADD(C[r + c * ldc], V_MUL(a, axj));
            }
        }
    }
}

/* COO: kernel_spmatmul_coo_N! / kernel_spmatmul_coo_T!
 * (src/matrix_coo/matrix_coo_kernels.jl:1-43).  One contribution per stored
 * entry, any storage order, no duplicate merging: C[out,c] += a*(B(in,c)*alpha). */
static void FN(coo)(int64_t nnz, const I *rowind, const I *colind, const V *val, int base,
                    int trans, int conjA, int64_t k, const V *B, int64_t ldb, int opB,
                    V *C, int64_t ldc, V alpha) {
    for (int64_t c = 0; c < k; ++c) {
        for (int64_t i = 0; i < nnz; ++i) {
            int64_t row = (int64_t)rowind[i] - base, col = (int64_t)colind[i] - base;
            int64_t out = trans ? col : row, in = trans ? row : col;
            V a = conjA ? V_CONJ(val[i]) : val[i];
            V axj = V_MUL(FN(getB)(B, ldb, opB, in, c), alpha);
            C[out + c * ldc] = V_ADD(C[out + c * ldc], V_MUL(a, axj));
        }
    }
}

/* mul!(C, op(A), op(B), alpha, beta) dispatch, following the method
 * generators src/matrix_csr/matrix_csr.jl:145-211,
 * src/matrix_csc/matrix_csc.jl:144-213 and src/matrix_coo/matrix_coo.jl:155-221:
 * beta pass first, then the N (opA == 0) or T kernel with CONJA = (opA == 2).
 * fmt: 0 CSR (p0 rowptr, p1 colval), 1 CSC (p0 colptr, p1 rowval),
 *      2 COO (p0 rowind, p1 colind). */
static int FN(mul)(int fmt, int opA, int64_t m, int64_t n, int64_t nnz,
                   const void *p0v, const void *p1v, const void *valv, int base,
                   int64_t k, const void *Bv, int64_t ldb, int opB,
                   void *Cv, int64_t ldc, const void *alphav, const void *betav, int nthreads) {
    const I *p0 = (const I *)p0v, *p1 = (const I *)p1v;
    const V *val = (const V *)valv, *B = (const V *)Bv;
    V *C = (V *)Cv;
    V alpha = *(const V *)alphav, beta = *(const V *)betav;
    int conjA = (opA == 2);
    int64_t rows_out = (opA == 0) ? m : n;
    FN(rmul_or_fill)(C, rows_out, k, ldc, beta);
    if (fmt == 0) {
        if (opA == 0) FN(gather)(m, p0, p1, val, base, conjA, k, B, ldb, opB, C, ldc, alpha, nthreads);
        else FN(scatter)(m, p0, p1, val, base, conjA, k, B, ldb, opB, C, ldc, alpha);
    } else if (fmt == 1) {
        if (opA == 0) FN(scatter)(n, p0, p1, val, base, conjA, k, B, ldb, opB, C, ldc, alpha);
        else FN(gather)(n, p0, p1, val, base, conjA, k, B, ldb, opB, C, ldc, alpha, nthreads);
    } else if (fmt == 2) {
        FN(coo)(nnz, p0, p1, val, base, opA != 0, conjA, k, B, ldb, opB, C, ldc, alpha);
    } else {
        return 1;
    }
    return 0;
}

/* |re + i im| without hypot's cost when the imaginary part is zero (real types). */
static inline double FN(absv)(double re, double im) { return im == 0.0 ? fabs(re) : hypot(re, im); }

/* The double-double contributions of outer entries [olo, ohi) (entries for COO) to
 * column c of the accumulators. */
static void FN(exact_range)(int fmt, int conjA, int trans, int64_t rows_out, int64_t c,
                            int64_t olo, int64_t ohi, const I *p0, const I *p1, const V *val, int base,
                            const V *B, int64_t ldb, int opB, dd *are, dd *aim, double *abssum) {
    for (int64_t o = olo; o < ohi; ++o) {
        int64_t jlo = (fmt == 2) ? o : (int64_t)p0[o] - base;
        int64_t jhi = (fmt == 2) ? o + 1 : (int64_t)p0[o + 1] - base;
        for (int64_t j = jlo; j < jhi; ++j) {
            int64_t row, col;
            if (fmt == 0) { row = o; col = (int64_t)p1[j] - base; }
            else if (fmt == 1) { row = (int64_t)p1[j] - base; col = o; }
            else { row = (int64_t)p0[j] - base; col = (int64_t)p1[j] - base; }
            int64_t out = trans ? col : row, in = trans ? row : col;
            double ar, ai, br, bi;
            V_TO_C(val[j], ar, ai);
            if (conjA) ai = -ai;
            V_TO_C(FN(getB)(B, ldb, opB, in, c), br, bi);
            int64_t t = out + c * rows_out;
            are[t] = dd_add_dd(are[t], two_prod(ar, br));
            are[t] = dd_add_dd(are[t], two_prod(-ai, bi));
            aim[t] = dd_add_dd(aim[t], two_prod(ar, bi));
            aim[t] = dd_add_dd(aim[t], two_prod(ai, br));
            abssum[t] += FN(absv)(ar, ai) * FN(absv)(br, bi);
        }
    }
}

/* Error oracle: the same product in double-double, with the per-output scale
 * |alpha| * sum_j |a_j||b_j| + |beta||C0| that the tolerance is relative to.
 * Outputs are doubles: yre/yim and scale, each rows_out x k column-major
 * (yim is ignored for real types).  Contributions are format-agnostic: every
 * stored entry adds a(out, in) * B(in, c) to output out.  Work is split over the
 * host threads where no two threads add into one output: over outer entries when
 * each outer entry owns its output (CSR N, CSC T/C), else over columns of B. */
static int FN(mul_exact)(int fmt, int opA, int64_t m, int64_t n, int64_t nnz,
                         const void *p0v, const void *p1v, const void *valv, int base,
                         int64_t k, const void *Bv, int64_t ldb, int opB,
                         const void *C0v, int64_t ldc0, const void *alphav, const void *betav,
                         double *yre, double *yim, double *scale) {
    const I *p0 = (const I *)p0v, *p1 = (const I *)p1v;
    const V *val = (const V *)valv, *B = (const V *)Bv;
    const V *C0 = (const V *)C0v;
    V alpha = *(const V *)alphav, beta = *(const V *)betav;
    int conjA = (opA == 2), trans = (opA != 0);
    int64_t rows_out = trans ? n : m;
    int64_t tot = rows_out * k;
    dd *are = (dd *)calloc((size_t)(tot > 0 ? tot : 1), sizeof(dd));
    dd *aim = (dd *)calloc((size_t)(tot > 0 ? tot : 1), sizeof(dd));
    double *abssum = (double *)calloc((size_t)(tot > 0 ? tot : 1), sizeof(double));
    if (!are || !aim || !abssum) { free(are); free(aim); free(abssum); return 2; }
    int64_t outer_n = (fmt == 0) ? m : n;
    int64_t cnt = (fmt == 2) ? nnz : outer_n;
    const int own_rows = (fmt == 0 && !trans) || (fmt == 1 && trans);
    /* small products stay on the calling thread (callers may check many at once) */
    const int big = (double)nnz * (double)(k > 0 ? k : 1) >= (double)(1 << 20);
    if (own_rows) {
        const int64_t step = 4096;
        for (int64_t c = 0; c < k; ++c) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) if (big)
#endif
            for (int64_t o = 0; o < cnt; o += step)
                FN(exact_range)(fmt, conjA, trans, rows_out, c, o, o + step < cnt ? o + step : cnt, p0, p1,
                                val, base, B, ldb, opB, are, aim, abssum);
        }
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) if (big)
#endif
        for (int64_t c = 0; c < k; ++c)
            FN(exact_range)(fmt, conjA, trans, rows_out, c, 0, cnt, p0, p1, val, base, B, ldb, opB, are, aim,
                            abssum);
    }
    double alr, ali, ber, bei;
    V_TO_C(alpha, alr, ali);
    V_TO_C(beta, ber, bei);
    int beta_one = V_EQ_ONE(beta), beta_zero = V_IS_ZERO(beta);
    for (int64_t c = 0; c < k; ++c) {
        for (int64_t r = 0; r < rows_out; ++r) {
            int64_t t = r + c * rows_out;
            /* alpha * acc */
            dd re = dd_add_dd(dd_mul_d(are[t], alr), dd_mul_d(aim[t], -ali));
            dd im = dd_add_dd(dd_mul_d(are[t], ali), dd_mul_d(aim[t], alr));
            double yr = 0.0, yi = 0.0, s = hypot(alr, ali) * abssum[t];
            if (!beta_zero) {
                V_TO_C(C0[r + c * ldc0], yr, yi);
                if (!beta_one) {
                    re = dd_add_dd(re, dd_add_dd(two_prod(yr, ber), two_prod(-yi, bei)));
                    im = dd_add_dd(im, dd_add_dd(two_prod(yr, bei), two_prod(yi, ber)));
                } else {
                    re = dd_add(re, yr);
                    im = dd_add(im, yi);
                }
                s += hypot(ber, bei) * hypot(yr, yi);
            }
            yre[t] = re.hi + re.lo;
            if (yim) yim[t] = im.hi + im.lo;
            scale[t] = s;
        }
    }
    free(are); free(aim); free(abssum);
    return 0;
}

/* Three-argument dot(x, op(A), y) = sum over stored entries of conj(x_l) * a * y_r,
 * following kernel_workgroup_dot_{csr,csc,coo}_{N,T}! (src/matrix_csr/matrix_csr_kernels.jl:47-131,
 * src/matrix_csc/matrix_csc_kernels.jl:47-131, src/matrix_coo/matrix_coo_kernels.jl:45-130)
 * and LinearAlgebra's dot(x::Number, a::Number, y::Number) = conj(x) * a * y: for an
 * entry (row, col), l = row and r = col for op = N, swapped for T/C (a conjugated for C).
 * *out gets the sum in the reference's arithmetic, terms in storage order (one of the
 * orders the reference's work items may take; exact for integers); out_re/out_im the
 * sum in double-double and out_scale sum |x_l||a||y_r|. */
static int FN(dot)(int fmt, int opA, int64_t m, int64_t n, int64_t nnz,
                   const void *p0v, const void *p1v, const void *valv, int base,
                   const void *xv, const void *yv, void *outv,
                   double *out_re, double *out_im, double *out_scale) {
    const I *p0 = (const I *)p0v, *p1 = (const I *)p1v;
    const V *val = (const V *)valv, *x = (const V *)xv, *y = (const V *)yv;
    int conjA = (opA == 2), trans = (opA != 0);
    int64_t outer_n = (fmt == 0) ? m : n;
    int64_t cnt = (fmt == 2) ? nnz : outer_n;
    V sum = V_ZERO;
    dd sre = {0.0, 0.0}, sim = {0.0, 0.0};
    double scale = 0.0;
    for (int64_t o = 0; o < cnt; ++o) {
        int64_t jlo = (fmt == 2) ? o : (int64_t)p0[o] - base;
        int64_t jhi = (fmt == 2) ? o + 1 : (int64_t)p0[o + 1] - base;
        for (int64_t j = jlo; j < jhi; ++j) {
            int64_t row, col;
            if (fmt == 0) { row = o; col = (int64_t)p1[j] - base; }
            else if (fmt == 1) { row = (int64_t)p1[j] - base; col = o; }
            else { row = (int64_t)p0[j] - base; col = (int64_t)p1[j] - base; }
            int64_t l = trans ? col : row, r = trans ? row : col;
            V a = conjA ? V_CONJ(val[j]) : val[j];
            sum = V_ADD(sum, V_MUL(V_MUL(V_CONJ(x[l]), a), y[r]));
            double xr, xi, ar, ai, yr, yi;
            V_TO_C(x[l], xr, xi);
            V_TO_C(a, ar, ai);
            V_TO_C(y[r], yr, yi);
            /* p = conj(x) a, exactly as double-double parts; then p * y */
            dd pr = dd_add_dd(two_prod(xr, ar), two_prod(xi, ai));
            dd pi = dd_add_dd(two_prod(xr, ai), two_prod(-xi, ar));
            sre = dd_add_dd(sre, dd_add_dd(dd_mul_d(pr, yr), dd_mul_d(pi, -yi)));
            sim = dd_add_dd(sim, dd_add_dd(dd_mul_d(pr, yi), dd_mul_d(pi, yr)));
            scale += hypot(xr, xi) * hypot(ar, ai) * hypot(yr, yi);
        }
    }
    *(V *)outv = sum;
    *out_re = sre.hi + sre.lo;
    *out_im = sim.hi + sim.lo;
    *out_scale = scale;
    return 0;
}

/* COO -> compressed conversion, following src/conversions/conversions.jl:282-323
 * (COO -> CSR) and :171-212 (COO -> CSC) with kernel_make_csr_keys! /
 * kernel_make_csc_keys! (src/conversions/conversion_kernels.jl:38-57):
 * key = major * minor_dim + minor, a stable sortperm of the keys, the three
 * gathers by perm, ptr[r] = searchsortedfirst(major_sorted, r) and
 * ptr[end] = nnz + 1 (in the index base).  Duplicates are kept, in input
 * order.  Keys are unsigned 64-bit (the reference computes them in Ti, which
 * wraps for Int32 once major_dim * minor_dim >= 2^31). */
static int FN(coo_to_compressed)(int colmajor, int64_t m, int64_t n, int64_t nnz,
                                 const void *rowindv, const void *colindv, const void *valv,
                                 int base, void *ptr_outv, void *idx_outv, void *val_outv) {
    const I *rowind = (const I *)rowindv, *colind = (const I *)colindv;
    const V *val = (const V *)valv;
    I *ptr_out = (I *)ptr_outv, *idx_out = (I *)idx_outv;
    V *val_out = (V *)val_outv;
    const I *major = colmajor ? colind : rowind;
    const I *minor = colmajor ? rowind : colind;
    int64_t major_n = colmajor ? n : m, minor_n = colmajor ? m : n;
    if (nnz <= 0) {
        for (int64_t r = 0; r <= major_n; ++r) ptr_out[r] = (I)base;
        return 0;
    }
    uint64_t *keys = (uint64_t *)malloc((size_t)nnz * sizeof(uint64_t));
    int64_t *perm = (int64_t *)malloc((size_t)nnz * sizeof(int64_t));
    int64_t *tmp = (int64_t *)malloc((size_t)nnz * sizeof(int64_t));
    if (!keys || !perm || !tmp) { free(keys); free(perm); free(tmp); return 2; }
    for (int64_t i = 0; i < nnz; ++i) {
        keys[i] = (uint64_t)((int64_t)major[i] - base) * (uint64_t)minor_n +
                  (uint64_t)((int64_t)minor[i] - base);
        perm[i] = i;
    }
    stable_sortperm(keys, perm, tmp, nnz);
    for (int64_t i = 0; i < nnz; ++i) {
        idx_out[i] = minor[perm[i]];
        val_out[i] = val[perm[i]];
    }
    /* searchsortedfirst over the sorted major indices, one query per major r */
    int64_t pos = 0;
    for (int64_t r = 0; r < major_n; ++r) {
        while (pos < nnz && (int64_t)major[perm[pos]] - base < r) ++pos;
        ptr_out[r] = (I)(pos + base);
    }
    ptr_out[major_n] = (I)(nnz + base);
    free(keys); free(perm); free(tmp);
    return 0;
}

/* Sums of COO matrices, following Base.:+ for GenericSparseMatrixCOO
 * (src/matrix_coo/matrix_coo.jl:300-385 A + B, :387-458 A + lambda*I, :460-575 the
 * transposed / adjoint pairs, A - B = A + (-B)): concatenate A's entries (indices swapped
 * when transposed, values conjugated when adjoint, negated for a subtraction), B's, then
 * the n_diag diagonal entries of lambda; keys col * m + row (kernel_make_csc_keys!,
 * src/conversions/conversion_kernels.jl:38-46; unsigned 64-bit here); a stable sortperm;
 * kernel_mark_unique_coo! and kernel_compact_coo! (src/matrix_coo/matrix_coo_kernels.jl:
 * 257-311: each run summed left to right in sorted order); then dropzeros (the entries whose
 * sum is zero removed, src/matrix_coo/matrix_coo.jl dropzeros).  ops: 0 N, 1 T, 2 C, | 4 to
 * negate.  Outputs hold room for nnz_a + nnz_b + n_diag entries; *kept gets the count. */
static int FN(coo_sum)(int64_t m, int64_t n, int64_t nnz_a, const void *ra, const void *ca, const void *va,
                       int op_a, int64_t nnz_b, const void *rb, const void *cb, const void *vb, int op_b,
                       int64_t n_diag, const void *lambdav, int base, void *row_outv, void *col_outv,
                       void *val_outv, int64_t *kept) {
    (void)n;
    const int64_t total = nnz_a + nnz_b + n_diag;
    I *row_out = (I *)row_outv, *col_out = (I *)col_outv;
    V *val_out = (V *)val_outv;
    *kept = 0;
    if (total <= 0) return 0;
    int64_t *rc = (int64_t *)malloc((size_t)total * 2 * sizeof(int64_t));
    V *vc = (V *)malloc((size_t)total * sizeof(V));
    uint64_t *keys = (uint64_t *)malloc((size_t)total * sizeof(uint64_t));
    int64_t *perm = (int64_t *)malloc((size_t)total * sizeof(int64_t));
    int64_t *tmp = (int64_t *)malloc((size_t)total * sizeof(int64_t));
    if (!rc || !vc || !keys || !perm || !tmp) { free(rc); free(vc); free(keys); free(perm); free(tmp); return 2; }
    int64_t e = 0;
    for (int w = 0; w < 2; ++w) {
        const int64_t cnt = w ? nnz_b : nnz_a;
        const I *r = (const I *)(w ? rb : ra), *c = (const I *)(w ? cb : ca);
        const V *v = (const V *)(w ? vb : va);
        const int op = (w ? op_b : op_a) & 3, neg = ((w ? op_b : op_a) & 4) != 0;
        for (int64_t i = 0; i < cnt; ++i, ++e) {
            const int64_t ri = (int64_t)r[i] - base, ci = (int64_t)c[i] - base;
            rc[2 * e] = op ? ci : ri;
            rc[2 * e + 1] = op ? ri : ci;
            V x = op == 2 ? V_CONJ(v[i]) : v[i];
            vc[e] = neg ? V_NEG(x) : x;
        }
    }
    for (int64_t d = 0; d < n_diag; ++d, ++e) {
        rc[2 * e] = rc[2 * e + 1] = d;
        vc[e] = *(const V *)lambdav;
    }
    for (int64_t i = 0; i < total; ++i) {
        keys[i] = (uint64_t)rc[2 * i + 1] * (uint64_t)m + (uint64_t)rc[2 * i];
        perm[i] = i;
    }
    stable_sortperm(keys, perm, tmp, total);
    int64_t out = 0;
    for (int64_t i = 0; i < total;) {
        V sum = vc[perm[i]];
        int64_t j = i + 1;
        while (j < total && keys[perm[j]] == keys[perm[i]]) sum = V_ADD(sum, vc[perm[j++]]);
        if (!V_IS_ZERO(sum)) {
            row_out[out] = (I)(rc[2 * perm[i]] + base);
            col_out[out] = (I)(rc[2 * perm[i] + 1] + base);
            val_out[out] = sum;
            ++out;
        }
        i = j;
    }
    *kept = out;
    free(rc); free(vc); free(keys); free(perm); free(tmp);
    return 0;
}

/* Sparse x sparse product, following kernel_count_nnz_spgemm_csr! / kernel_spgemm_csr!
 * (src/matrix_csr/matrix_csr_kernels.jl:250-343, method src/matrix_csr/matrix_csr.jl:498-556)
 * and kernel_count_nnz_spgemm_csc! / kernel_spgemm_csc! (src/matrix_csc/matrix_csc_kernels.jl:
 * 255-345, method src/matrix_csc/matrix_csc.jl:500-560).  fmt 0 (CSR): for each row i of A,
 * for each stored A[i,k] in storage order, for each stored B[k,j] in storage order,
 * acc[j] += A[i,k] * B[k,j]; fmt 1 (CSC): for each column j of B, for each stored B[k,j],
 * for each stored A[i,k], acc[i] += A[i,k] * B[k,j].  acc starts at zero; every position
 * reached is stored (zero sums included), in increasing index order.  m x kk times kk x n.
 * Outputs: ptr_out (outer + 1, index base), and when idx_out is not NULL the indices and
 * values (room for `cap` entries); *nnz_out gets the entry count. */
static int FN(spgemm)(int fmt, int64_t m, int64_t kk, int64_t n, const void *pav, const void *iav,
                      const void *vav, const void *pbv, const void *ibv, const void *vbv, int base,
                      void *ptr_outv, void *idx_outv, void *val_outv, int64_t cap, int64_t *nnz_out) {
    (void)kk;
    const I *pa = (const I *)pav, *ia = (const I *)iav, *pb = (const I *)pbv, *ib = (const I *)ibv;
    const V *va = (const V *)vav, *vb = (const V *)vbv;
    I *ptr_out = (I *)ptr_outv, *idx_out = (I *)idx_outv;
    V *val_out = (V *)val_outv;
    /* the outer loop runs over P's outer entries, the inner over Q's: CSR P = A, Q = B;
     * CSC P = B, Q = A */
    const int csr = fmt == 0;
    const int64_t outer_n = csr ? m : n, width = csr ? n : m;
    const I *pp = csr ? pa : pb, *pi = csr ? ia : ib, *qp = csr ? pb : pa, *qi = csr ? ib : ia;
    const V *pv = csr ? va : vb, *qv = csr ? vb : va;
    V *acc = (V *)malloc((size_t)(width > 0 ? width : 1) * sizeof(V));
    unsigned char *seen = (unsigned char *)calloc((size_t)(width > 0 ? width : 1), 1);
    if (!acc || !seen) { free(acc); free(seen); return 2; }
    for (int64_t j = 0; j < width; ++j) acc[j] = V_ZERO;
    int64_t out = 0;
    for (int64_t o = 0; o < outer_n; ++o) {
        ptr_out[o] = (I)(out + base);
        for (int64_t e = (int64_t)pp[o] - base; e < (int64_t)pp[o + 1] - base; ++e) {
            const int64_t k = (int64_t)pi[e] - base;
            for (int64_t f = (int64_t)qp[k] - base; f < (int64_t)qp[k + 1] - base; ++f) {
                const int64_t j = (int64_t)qi[f] - base;
                const V prod = csr ? V_MUL(pv[e], qv[f]) : V_MUL(qv[f], pv[e]);
                acc[j] = V_ADD(acc[j], prod);
                seen[j] = 1;
            }
        }
        for (int64_t j = 0; j < width; ++j) {
            if (!seen[j]) continue;
            if (idx_out && out < cap) {
                idx_out[out] = (I)(j + base);
                val_out[out] = acc[j];
            }
            ++out;
            seen[j] = 0;
            acc[j] = V_ZERO;
        }
    }
    ptr_out[outer_n] = (I)(out + base);
    *nnz_out = out;
    free(acc); free(seen);
    return 0;
}

/* Sum of two compressed matrices of one format, following kernel_count_nnz_per_row_csr! and
 * kernel_merge_csr! (src/matrix_csr/matrix_csr_kernels.jl:146-248; the CSC kernels at
 * src/matrix_csc/matrix_csc_kernels.jl:146-250) inside Base.:+ (src/matrix_csr/matrix_csr.jl:
 * 290-356, src/matrix_csc/matrix_csc.jl:292-357): per outer entry a two-pointer walk over A's and
 * B's stored entries in storage order -- the smaller index first, equal indices summed a + b --
 * then dropzeros.  neg_b negates B's values (A - B = A + (-B), src/core.jl:91).  Outputs have
 * room for nnz_a + nnz_b entries. */
static int FN(compressed_add)(int64_t outer_n, const void *pav, const void *iav, const void *vav, const void *pbv,
                              const void *ibv, const void *vbv, int neg_b, int base, void *ptr_outv, void *idx_outv,
                              void *val_outv, int64_t *nnz_out) {
    const I *pa = (const I *)pav, *ia = (const I *)iav, *pb = (const I *)pbv, *ib = (const I *)ibv;
    const V *va = (const V *)vav, *vb = (const V *)vbv;
    I *ptr_out = (I *)ptr_outv, *idx_out = (I *)idx_outv;
    V *val_out = (V *)val_outv;
    int64_t w = 0;
    for (int64_t o = 0; o < outer_n; ++o) {
        ptr_out[o] = (I)(w + base);
        int64_t a = (int64_t)pa[o] - base, ae = (int64_t)pa[o + 1] - base;
        int64_t b = (int64_t)pb[o] - base, be = (int64_t)pb[o + 1] - base;
        while (a < ae || b < be) {
            I idx;
            V v;
            if (a < ae && b < be && ia[a] == ib[b]) {
                idx = ia[a];
                v = V_ADD(va[a], neg_b ? V_NEG(vb[b]) : vb[b]);
                ++a; ++b;
            } else if (b >= be || (a < ae && ia[a] < ib[b])) {
                idx = ia[a]; v = va[a]; ++a;
            } else {
                idx = ib[b]; v = neg_b ? V_NEG(vb[b]) : vb[b]; ++b;
            }
            if (V_IS_ZERO(v)) continue;  /* dropzeros */
            idx_out[w] = idx;
            val_out[w] = v;
            ++w;
        }
    }
    ptr_out[outer_n] = (I)(w + base);
    *nnz_out = w;
    return 0;
}

/* A + lambda*I for a square compressed matrix, following kernel_count_diag_entries_csr! and
 * kernel_add_uniformscaling_csr! (src/matrix_csr/matrix_csr_kernels.jl:446-507; the CSC kernels
 * at src/matrix_csc/matrix_csc_kernels.jl:446-510) inside Base.:+ (src/matrix_csr/matrix_csr.jl:
 * 358-402): an outer entry without a stored diagonal gets one more entry; the walk copies the
 * entries, adds lambda to every stored diagonal, and inserts (o, lambda) before the first entry
 * past the diagonal or at the end.  No dropzeros.  Writes stay inside each entry's counted room
 * (the reference writes past it for a row whose diagonal follows a larger index). */
static int FN(compressed_add_diag)(int64_t n, const void *pav, const void *iav, const void *vav, const void *lamv,
                                   int base, void *ptr_outv, void *idx_outv, void *val_outv, int64_t *nnz_out) {
    const I *pa = (const I *)pav, *ia = (const I *)iav;
    const V *va = (const V *)vav;
    const V lam = *(const V *)lamv;
    I *ptr_out = (I *)ptr_outv, *idx_out = (I *)idx_outv;
    V *val_out = (V *)val_outv;
    int64_t w0 = 0;
    for (int64_t o = 0; o < n; ++o) {
        const int64_t b = (int64_t)pa[o] - base, e = (int64_t)pa[o + 1] - base;
        int found = 0;
        for (int64_t j = b; j < e; ++j)
            if ((int64_t)ia[j] - base == o) { found = 1; break; }
        const int64_t end = w0 + (e - b) + (found ? 0 : 1);
        ptr_out[o] = (I)(w0 + base);
        int64_t w = w0;
        int written = 0;
        for (int64_t j = b; j < e; ++j) {
            const int64_t col = (int64_t)ia[j] - base;
            if (!written && col > o) {
                if (w < end) { idx_out[w] = (I)(o + base); val_out[w] = lam; }
                ++w;
                written = 1;
            }
            if (w < end) {
                idx_out[w] = ia[j];
                if (col == o) { val_out[w] = V_ADD(va[j], lam); written = 1; }
                else val_out[w] = va[j];
            }
            ++w;
        }
        if (!written && w < end) { idx_out[w] = (I)(o + base); val_out[w] = lam; }
        w0 = end;
    }
    ptr_out[n] = (I)(w0 + base);
    *nnz_out = w0;
    return 0;
}

/* Compressed -> COO expansion: kernel_csr_to_coo! / kernel_csc_to_coo!
 * (src/conversions/conversion_kernels.jl:2-35).  Every stored entry of outer
 * o gets major index o (in the index base); minor indices and values copy. */
static int FN(compressed_to_coo)(int colmajor, int64_t m, int64_t n, int64_t nnz,
                                 const void *ptrv, const void *idxv, const void *valv, int base,
                                 void *rowind_outv, void *colind_outv, void *val_outv) {
    const I *ptr = (const I *)ptrv, *idx = (const I *)idxv;
    const V *val = (const V *)valv;
    I *rowind_out = (I *)rowind_outv, *colind_out = (I *)colind_outv;
    V *val_out = (V *)val_outv;
    int64_t outer_n = colmajor ? n : m;
    (void)nnz;
    for (int64_t o = 0; o < outer_n; ++o) {
        for (int64_t j = (int64_t)ptr[o] - base; j < (int64_t)ptr[o + 1] - base; ++j) {
            I major = (I)(o + base);
            if (colmajor) { rowind_out[j] = idx[j]; colind_out[j] = major; }
            else { rowind_out[j] = major; colind_out[j] = idx[j]; }
            val_out[j] = val[j];
        }
    }
    return 0;
}

#undef FN
