/*
 * CPU oracle for the sparse x dense mul! path and the COO <-> CSR/CSC
 * conversions of GenericSparseArrays.jl.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library, and there only to check results
 * (or as the timed CPU restatement of the reference).  The CUDA library never
 * links or calls it.
 *
 * It restates, in plain C, the reference's KernelAbstractions kernels and
 * method bodies (each function in gsa_oracle_impl.h cites the reference
 * file:line it follows).  Arithmetic follows Julia: no FMA contraction (build
 * with -ffp-contract=off), complex products by the textbook formula, and
 * wrapping integer arithmetic for Int32/Int64 values.
 *
 * Parity pin: the reference (Julia) cannot run on either machine of this
 * build, so the restatement is pinned against the known-answer fixtures the
 * reference's own tests and docs hold (tests/golden/) and cross-checked
 * against scipy.sparse, which stands in for SparseArrays.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { float re, im; } cf32;
typedef struct { double re, im; } cf64;

/* ---- double-double helpers (error oracle only) ---------------------------- */
typedef struct { double hi, lo; } dd;

static inline dd two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    dd r = {s, (a - (s - bb)) + (b - bb)};
    return r;
}
static inline dd two_prod(double a, double b) {
    double p = a * b;
    dd r = {p, fma(a, b, -p)};
    return r;
}
static inline dd dd_add(dd a, double b) {
    dd s = two_sum(a.hi, b);
    s.lo += a.lo;
    return two_sum(s.hi, s.lo);
}
static inline dd dd_add_dd(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return two_sum(s.hi, s.lo);
}
static inline dd dd_mul_d(dd a, double b) {
    dd p = two_prod(a.hi, b);
    p.lo += a.lo * b;
    return two_sum(p.hi, p.lo);
}

/* ---- stable sortperm by 64-bit key (bottom-up merge sort) ----------------- */
static void stable_sortperm(const uint64_t *keys, int64_t *perm, int64_t *tmp, int64_t n) {
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n;
            int64_t hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t a = lo, b = mid, o = lo;
            while (a < mid && b < hi) {
                if (keys[perm[b]] < keys[perm[a]]) tmp[o++] = perm[b++];
                else tmp[o++] = perm[a++];
            }
            while (a < mid) tmp[o++] = perm[a++];
            while (b < hi) tmp[o++] = perm[b++];
        }
        memcpy(perm, tmp, (size_t)n * sizeof(int64_t));
    }
}

/* ---- per-type arithmetic ----------------------------------------------- */
static inline cf32 cf32_mul(cf32 a, cf32 b) {
    cf32 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cf64 cf64_mul(cf64 a, cf64 b) {
    cf64 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cf32 cf32_add(cf32 a, cf32 b) { cf32 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf64 cf64_add(cf64 a, cf64 b) { cf64 r = {a.re + b.re, a.im + b.im}; return r; }
static inline cf32 cf32_conj(cf32 a) { cf32 r = {a.re, -a.im}; return r; }
static inline cf64 cf64_conj(cf64 a) { cf64 r = {a.re, -a.im}; return r; }
static inline cf32 cf32_neg(cf32 a) { cf32 r = {-a.re, -a.im}; return r; }
static inline cf64 cf64_neg(cf64 a) { cf64 r = {-a.re, -a.im}; return r; }
static const cf32 cf32_zero = {0.0f, 0.0f};
static const cf64 cf64_zero = {0.0, 0.0};

#define I32_ADD(a, b) ((int32_t)((uint32_t)(a) + (uint32_t)(b)))
#define I32_MUL(a, b) ((int32_t)((uint32_t)(a) * (uint32_t)(b)))
#define I64_ADD(a, b) ((int64_t)((uint64_t)(a) + (uint64_t)(b)))
#define I64_MUL(a, b) ((int64_t)((uint64_t)(a) * (uint64_t)(b)))

/* Instantiate the body for every (value, index) pair. */
/* float */
#define V float
#define V_ZERO 0.0f
#define V_ADD(a, b) ((a) + (b))
#define V_MUL(a, b) ((a) * (b))
#define V_CONJ(a) (a)
#define V_NEG(a) (-(a))
#define V_EQ_ONE(a) ((a) == 1.0f)
#define V_IS_ZERO(a) ((a) == 0.0f)
#define V_TO_C(a, r, i) do { (r) = (double)(a); (i) = 0.0; } while (0)
#define I int32_t
#define SUFFIX f32_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX f32_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V
#undef V_ZERO
#undef V_EQ_ONE
#undef V_IS_ZERO

/* double */
#define V double
#define V_ZERO 0.0
#define V_EQ_ONE(a) ((a) == 1.0)
#define V_IS_ZERO(a) ((a) == 0.0)
#define I int32_t
#define SUFFIX f64_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX f64_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V
#undef V_ZERO
#undef V_ADD
#undef V_MUL
#undef V_CONJ
#undef V_NEG
#undef V_EQ_ONE
#undef V_IS_ZERO
#undef V_TO_C

/* ComplexF32 */
#define V cf32
#define V_ZERO cf32_zero
#define V_ADD(a, b) cf32_add((a), (b))
#define V_MUL(a, b) cf32_mul((a), (b))
#define V_CONJ(a) cf32_conj(a)
#define V_NEG(a) cf32_neg(a)
#define V_EQ_ONE(a) ((a).re == 1.0f && (a).im == 0.0f)
#define V_IS_ZERO(a) ((a).re == 0.0f && (a).im == 0.0f)
#define V_TO_C(a, r, i) do { (r) = (double)(a).re; (i) = (double)(a).im; } while (0)
#define I int32_t
#define SUFFIX c32_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX c32_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V
#undef V_ZERO
#undef V_ADD
#undef V_MUL
#undef V_CONJ
#undef V_NEG
#undef V_EQ_ONE
#undef V_IS_ZERO
#undef V_TO_C

/* ComplexF64 */
#define V cf64
#define V_ZERO cf64_zero
#define V_ADD(a, b) cf64_add((a), (b))
#define V_MUL(a, b) cf64_mul((a), (b))
#define V_CONJ(a) cf64_conj(a)
#define V_NEG(a) cf64_neg(a)
#define V_EQ_ONE(a) ((a).re == 1.0 && (a).im == 0.0)
#define V_IS_ZERO(a) ((a).re == 0.0 && (a).im == 0.0)
#define V_TO_C(a, r, i) do { (r) = (a).re; (i) = (a).im; } while (0)
#define I int32_t
#define SUFFIX c64_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX c64_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V
#undef V_ZERO
#undef V_ADD
#undef V_MUL
#undef V_CONJ
#undef V_NEG
#undef V_EQ_ONE
#undef V_IS_ZERO
#undef V_TO_C

/* Int32 values (wrapping, as Julia's Int32 arithmetic) */
#define V int32_t
#define V_ZERO 0
#define V_ADD(a, b) I32_ADD(a, b)
#define V_MUL(a, b) I32_MUL(a, b)
#define V_CONJ(a) (a)
#define V_NEG(a) ((int32_t)(0u - (uint32_t)(a)))
#define V_EQ_ONE(a) ((a) == 1)
#define V_IS_ZERO(a) ((a) == 0)
#define V_TO_C(a, r, i) do { (r) = (double)(a); (i) = 0.0; } while (0)
#define I int32_t
#define SUFFIX i32_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX i32_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V
#undef V_ZERO
#undef V_ADD
#undef V_MUL

/* Int64 values */
#define V int64_t
#define V_ZERO 0
#define V_ADD(a, b) I64_ADD(a, b)
#define V_MUL(a, b) I64_MUL(a, b)
#undef V_NEG
#define V_NEG(a) ((int64_t)(0ull - (uint64_t)(a)))
#define I int32_t
#define SUFFIX i64_i32
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#define I int64_t
#define SUFFIX i64_i64
#include "gsa_oracle_impl.h"
#undef I
#undef SUFFIX
#undef V

/* ---- exported dispatch ---------------------------------------------------
 * dtype: 0 Float32, 1 Float64, 2 ComplexF32, 3 ComplexF64, 4 Int32, 5 Int64
 * itype: 0 Int32, 1 Int64
 * Same codes as include/gsa.h.  Every function returns 0 on success. */

#define DISPATCH(FNAME, ...)                                                        \
    switch (dtype * 2 + itype) {                                                   \
    case 0: return FNAME##_f32_i32(__VA_ARGS__);                                  \
    case 1: return FNAME##_f32_i64(__VA_ARGS__);                                  \
    case 2: return FNAME##_f64_i32(__VA_ARGS__);                                  \
    case 3: return FNAME##_f64_i64(__VA_ARGS__);                                  \
    case 4: return FNAME##_c32_i32(__VA_ARGS__);                                  \
    case 5: return FNAME##_c32_i64(__VA_ARGS__);                                  \
    case 6: return FNAME##_c64_i32(__VA_ARGS__);                                  \
    case 7: return FNAME##_c64_i64(__VA_ARGS__);                                  \
    case 8: return FNAME##_i32_i32(__VA_ARGS__);                                  \
    case 9: return FNAME##_i32_i64(__VA_ARGS__);                                  \
    case 10: return FNAME##_i64_i32(__VA_ARGS__);                                 \
    case 11: return FNAME##_i64_i64(__VA_ARGS__);                                 \
    default: return 3;                                                            \
    }

int oracle_mul(int fmt, int opA, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
               const void *p0, const void *p1, const void *val, int base,
               int64_t k, const void *B, int64_t ldb, int opB,
               void *C, int64_t ldc, const void *alpha, const void *beta, int nthreads) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(mul, fmt, opA, m, n, nnz, p0, p1, val, base, k, B, ldb, opB, C, ldc, alpha, beta,
             nthreads)
}

int oracle_mul_exact(int fmt, int opA, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                     const void *p0, const void *p1, const void *val, int base,
                     int64_t k, const void *B, int64_t ldb, int opB,
                     const void *C0, int64_t ldc0, const void *alpha, const void *beta,
                     double *yre, double *yim, double *scale) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(mul_exact, fmt, opA, m, n, nnz, p0, p1, val, base, k, B, ldb, opB, C0, ldc0,
             alpha, beta, yre, yim, scale)
}

int oracle_dot(int fmt, int opA, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
               const void *p0, const void *p1, const void *val, int base, const void *x,
               const void *y, void *out, double *out_re, double *out_im, double *out_scale) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(dot, fmt, opA, m, n, nnz, p0, p1, val, base, x, y, out, out_re, out_im, out_scale)
}

int oracle_coo_to_compressed(int colmajor, int dtype, int itype, int64_t m, int64_t n,
                             int64_t nnz, const void *rowind, const void *colind,
                             const void *val, int base, void *ptr_out, void *idx_out,
                             void *val_out) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(coo_to_compressed, colmajor, m, n, nnz, rowind, colind, val, base, ptr_out,
             idx_out, val_out)
}

int oracle_compressed_to_coo(int colmajor, int dtype, int itype, int64_t m, int64_t n,
                             int64_t nnz, const void *ptr, const void *idx, const void *val,
                             int base, void *rowind_out, void *colind_out, void *val_out) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(compressed_to_coo, colmajor, m, n, nnz, ptr, idx, val, base, rowind_out,
             colind_out, val_out)
}

int oracle_coo_sum(int dtype, int itype, int64_t m, int64_t n, int64_t nnz_a, const void *ra, const void *ca,
                   const void *va, int op_a, int64_t nnz_b, const void *rb, const void *cb, const void *vb,
                   int op_b, int64_t n_diag, const void *lambda, int base, void *row_out, void *col_out,
                   void *val_out, int64_t *kept) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(coo_sum, m, n, nnz_a, ra, ca, va, op_a, nnz_b, rb, cb, vb, op_b, n_diag, lambda, base, row_out,
             col_out, val_out, kept)
}

int oracle_spgemm(int fmt, int dtype, int itype, int64_t m, int64_t kk, int64_t n, const void *pa, const void *ia,
                  const void *va, const void *pb, const void *ib, const void *vb, int base, void *ptr_out,
                  void *idx_out, void *val_out, int64_t cap, int64_t *nnz_out) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(spgemm, fmt, m, kk, n, pa, ia, va, pb, ib, vb, base, ptr_out, idx_out, val_out, cap, nnz_out)
}

int oracle_compressed_add(int dtype, int itype, int64_t outer_n, const void *pa, const void *ia, const void *va,
                          const void *pb, const void *ib, const void *vb, int neg_b, int base, void *ptr_out,
                          void *idx_out, void *val_out, int64_t *nnz_out) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(compressed_add, outer_n, pa, ia, va, pb, ib, vb, neg_b, base, ptr_out, idx_out, val_out, nnz_out)
}

int oracle_compressed_add_diag(int dtype, int itype, int64_t n, const void *pa, const void *ia, const void *va,
                               const void *lam, int base, void *ptr_out, void *idx_out, void *val_out,
                               int64_t *nnz_out) {
    if (dtype < 0 || dtype > 5 || itype < 0 || itype > 1) return 3;
    DISPATCH(compressed_add_diag, n, pa, ia, va, lam, base, ptr_out, idx_out, val_out, nnz_out)
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
