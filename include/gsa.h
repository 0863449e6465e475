/*
 * gsa.h -- C ABI of libgsa, the GB300 (sm_103a) library behind the sparse x dense
 * mul! path of GenericSparseArrays.jl and the COO -> CSR/CSC conversions that
 * feed it.
 *
 * Every entry point takes plain device pointers and sizes, runs asynchronously on
 * the caller's CUDA stream and returns a status code (GSA_OK == 0).  The library
 * never frees caller buffers.  gsa_last_error_string() gives a message for the
 * last failing call on the calling host thread.
 *
 * Conventions shared by all entry points
 *   dtype   element type of values and dense operands (gsa_dtype)
 *   itype   index type of pointer and index arrays (gsa_itype)
 *   base    index base of every index/pointer array: 1 for Julia's 1-based
 *           buffers (rowptr[0] == 1), 0 for C-style buffers
 *   alpha, beta  HOST pointers to one value of type dtype (complex: re, im)
 *   stream  a cudaStream_t (NULL = legacy default stream)
 *   Buffers must be aligned to their element size (complex: 2 x the real size).
 *
 * Dense operands are column-major (Julia's layout).  op(B) is given by its
 * parent buffer: opB == GSA_OP_N reads B(i, c) = B[i + c*ldb]; GSA_OP_T and
 * GSA_OP_C read B(i, c) = B[c + i*ldb] (GSA_OP_C conjugated), i.e. the parent
 * is the k x rows(op(B)) matrix that Julia's Transpose/Adjoint wraps.
 *
 * Workspace: entry points that need scratch take (workspace, workspace_bytes).
 * Pass workspace == NULL to let the library take it from the stream-ordered
 * pool (cudaMallocAsync / cudaFreeAsync on the same stream); otherwise pass at
 * least the size the matching *_workspace_size function returns.  A caller
 * workspace must not be used by another call that overlaps on the GPU.
 */
#ifndef GSA_H
#define GSA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GSA_OK = 0,
    GSA_ERR_INVALID_ARG = 1,   /* bad pointer, size, enum or alignment: ArgumentError */
    GSA_ERR_DIM = 2,           /* sizes of A, B, C do not agree: DimensionMismatch */
    GSA_ERR_UNSUPPORTED = 3,   /* dtype/itype/format combination not provided */
    GSA_ERR_CUDA = 4,          /* a CUDA launch or runtime call failed */
    GSA_ERR_ALLOC = 5,         /* stream-ordered workspace allocation failed */
    GSA_ERR_STRUCTURE = 6,     /* validator found a malformed matrix */
    GSA_ERR_TIMEOUT = 7        /* a bounded device-side wait gave up */
} gsa_status;

typedef enum {
    GSA_F32 = 0, GSA_F64 = 1, GSA_C32 = 2, GSA_C64 = 3, GSA_I32 = 4, GSA_I64 = 5
} gsa_dtype;

typedef enum { GSA_IDX32 = 0, GSA_IDX64 = 1 } gsa_itype;

/* op(A) / op(B): identity, transpose, adjoint (conjugate transpose). */
typedef enum { GSA_OP_N = 0, GSA_OP_T = 1, GSA_OP_C = 2 } gsa_op;

/* Gather kernel selection for the row-gather paths (CSR N, CSC T). */
typedef enum {
    GSA_ALGO_AUTO = 0,     /* library choice: row blocks -- per warp of 32 rows (columns
                              for the scatter directions), 1..32 lanes per row from the
                              rows' average length; no workspace */
    GSA_ALGO_MERGE = 1,    /* one CTA per merge-path tile (any row-length mix); gather and
                              scatter */
    GSA_ALGO_VECTOR = 2,   /* gather: a group of threads per row (short, even rows);
                              scatter with one right-hand side: a thread per outer entry,
                              products near the CTA's outer range (a band) summed in a
                              shared-memory window, one atomic per touched row; with
                              several right-hand sides as AUTO */
    GSA_ALGO_PIPE = 3      /* gather: persistent merge-path runs with bulk-copy double
                              buffering (one right-hand side); scatter: as AUTO */
} gsa_algo;

/* Tuning keys for gsa_set_tuning / gsa_get_tuning. */
typedef enum {
    GSA_TUNE_PIPE_THREADS = 1, /* threads per CTA of the pipelined SpMV: 256 or 512 */
    GSA_TUNE_SPMM_COLUMNS = 2, /* right-hand-side columns a thread accumulates in the default
                                  gather with k > 1: 0 (by value size), 1, 2, 4 or 8 */
    GSA_TUNE_PLAN_ORDER = 3,   /* 0: a planned gather runs in the plan's bin order where the
                                  plan has one and the product is FP64-bound (ComplexF64, or
                                  Float64 with several right-hand sides); 1: always in natural
                                  row order; 2: in the bin order for every Float64 / ComplexF64
                                  product whose plan has one */
    GSA_TUNE_STAGE_ROWS = 5,   /* 1: in the default gather with one right-hand side, Float32 /
                                  Float64 values and Int32 indices, warps of thread-per-row
                                  rows copy their contiguous entry span into shared memory with
                                  16-byte loads before summing (measured slower on GB300: a
                                  second memory round trip before the gathers); 2: each lane
                                  reads its own row in aligned 16-byte pieces into registers
                                  (4-5 % faster on rows of about 4 entries, slower on the
                                  Float64 Laplacian); 0 (default): direct loads */
    GSA_TUNE_X_PAIRS = 6,      /* 1 (default): with Float64 values, several right-hand sides and a
                                  row-major B (unit column stride, even row stride, 16-byte
                                  aligned), a thread of 4 or 8 columns reads its columns of one
                                  row of B two at a time with 16-byte loads; 0: one load per
                                  column */
    GSA_TUNE_SORT_STAGED = 7,  /* 1 (default): where rows average at most 8 entries, the
                                  conversions' bucket sort runs its row pass as one CTA per SM
                                  that copies its next bucket into shared memory (cp.async)
                                  while it sorts the current one; 0: two CTAs per SM that read
                                  their buckets as they go.  Same output either way */
    GSA_TUNE_WAIT_LIMIT = 4    /* polls a bounded device-side wait (the pipelined SpMV's
                                  mbarrier waits for its bulk copies) makes before it gives
                                  up, sets the device error word and returns: default
                                  16777216; 0 gives up at once (the timeout path, for tests) */
} gsa_tune_key;

/* ---- library ------------------------------------------------------------ */

/* Version as major*10000 + minor*100 + patch. */
int gsa_version(void);

/* Message for the last non-OK status returned on this host thread. */
const char *gsa_last_error_string(void);

/* Process-wide kernel tuning (no counterpart in the reference): set a key to a
 * value (GSA_ERR_INVALID_ARG if either is unknown), or read it back (-1 for an
 * unknown key).  Affects calls issued afterwards. */
int gsa_set_tuning(int key, int value);
int gsa_get_tuning(int key);

/* Profiling hook (no counterpart in the reference, which has no tracing): when set, the
 * library records `before` and `after` (cudaEvent_t) on the call's stream right around the
 * main compute kernel of each following call from this host thread -- the row-block,
 * merge-path, vector or pipelined gather, the scatter, the COO kernel, the grouped kernel,
 * or the whole sort of a conversion.  Pass
 * NULL, NULL to switch it off. */
void gsa_set_kernel_timer(void *before, void *after);

/* ---- sparse x dense mul! --------------------------------------------------
 * C = beta*C + alpha * op(A) * op(B), with C (rows(op(A)) x k, column-major,
 * leading dimension ldc).  beta == 0 never reads C (NaN in C is overwritten),
 * beta == 1 skips the scaling, as LinearAlgebra._rmul_or_fill! does before
 * the reference's kernels.  m x n is the stored (parent) size of A, nnz the
 * number of stored entries.  B and C must not overlap.
 */

/* Replaces the mul! methods generated at src/matrix_csr/matrix_csr.jl:145-211
 * (kernels kernel_spmatmul_csr_N! / _T!, src/matrix_csr/matrix_csr_kernels.jl:1-45).
 * opA == N gathers along rows; T/C scatter (CSR-T, atomics). */
int gsa_csr_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowptr, const void *colval, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta, int algo, void *workspace,
                size_t workspace_bytes);

/* Replaces src/matrix_csc/matrix_csc.jl:144-213 (kernels kernel_spmatmul_csc_N! /
 * _T!, src/matrix_csc/matrix_csc_kernels.jl:1-45).  opA == N scatters along
 * columns; T/C gather (the CSR-N kernel on the stored structure). */
int gsa_csc_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *colptr, const void *rowval, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta, int algo, void *workspace,
                size_t workspace_bytes);

/* Replaces src/matrix_coo/matrix_coo.jl:155-221 (kernels kernel_spmatmul_coo_N! /
 * _T!, src/matrix_coo/matrix_coo_kernels.jl:1-43).  Any storage order and
 * duplicates are accepted; runs of equal output rows are reduced in registers
 * before the atomics (warps without such a run, as in a COO of random order, go
 * straight to the atomics).  Needs no workspace. */
int gsa_coo_mul(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowind, const void *colind, const void *nzval, int base, int opA,
                int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                const void *alpha, const void *beta);

/* C += A for a dense m x n column-major C (leading dimension ldc): the kernel of `A + B`
 * with a dense B (src/core.jl:66-88 -- C = copy(B), then _add_sparse_to_dense!, kernels
 * kernel_add_sparse_to_dense_{csr,csc,coo}!, e.g. src/matrix_csr/matrix_csr_kernels.jl:133-145).
 * format: 0 CSR (p0 rowptr, p1 colval), 1 CSC (colptr, rowval), 2 COO (rowind, colind).
 * Duplicate entries add up; entries outside the matrix are skipped. */
int gsa_add_to_dense(void *stream, int format, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                     const void *p0, const void *p1, const void *nzval, int base, void *C, int64_t ldc);

/* dropzeros (src/matrix_csr/matrix_csr.jl:649-745, kernels kernel_count_nonzeros_csr! /
 * kernel_dropzeros_csr! at src/matrix_csr/matrix_csr_kernels.jl:409-443, and the CSC / COO
 * methods): the stored entries that are not zero, in storage order.  Two calls on ONE
 * workspace of gsa_dropzeros_workspace_size(nnz) bytes: _count finds the kept entries'
 * positions and returns their count on the host (synchronizes the stream); the caller
 * allocates the outputs; _copy writes them -- for CSR/CSC p0_out is the new pointer array
 * (outer_n + 1, same base) and p1_out/val_out the kept indices and values, for COO
 * p0_out/p1_out/val_out the kept (rowind, colind, nzval).  At most 2^32 - 2 entries. */
size_t gsa_dropzeros_workspace_size(int64_t nnz);
int gsa_dropzeros_count(void *stream, int dtype, int64_t nnz, const void *nzval, void *workspace,
                        size_t workspace_bytes, int64_t *kept);
int gsa_dropzeros_copy(void *stream, int format, int dtype, int itype, int64_t outer_n, int64_t nnz,
                       const void *p0, const void *p1, const void *nzval, int base, const void *workspace,
                       void *p0_out, void *p1_out, void *val_out);

/* Sums of COO matrices -- Base.:+ for GenericSparseMatrixCOO: A + B
 * (src/matrix_coo/matrix_coo.jl:300-385), A + λI (:387-458) and the transposed / adjoint
 * pairs and A - B (:460-575), kernels kernel_mark_unique_coo! / kernel_compact_coo!
 * (src/matrix_coo/matrix_coo_kernels.jl:257-311) and the dropzeros that ends each of them.
 * The result is m x n: the entries of source a (nnz_a entries), then of source b (nnz_b,
 * may be 0), then n_diag diagonal entries (i, i), i = 1..n_diag, of value *lambda (the
 * dtype's type, host memory; NULL allowed when n_diag = 0).  op_a / op_b: GSA_OP_N, T (row
 * and column indices swapped) or C (swapped and conjugated), optionally OR'ed with
 * GSA_SUM_NEGATE (values negated: A - B = A + (-B)).  Entries at the same (row, col) are
 * summed left to right in that order; sums that are zero are dropped; the output is in
 * column-major order (sorted by column, then row), as the reference's column-major keys
 * give it.  Two calls on ONE workspace of gsa_coo_sum_workspace_size(dtype, m, n, nnz_a + nnz_b +
 * n_diag) bytes: _count sorts and sums, returns the result's entry count on the host
 * (synchronizes the stream); the caller allocates the outputs (kept entries each); _copy,
 * given the same m, n, base, total = nnz_a + nnz_b + n_diag and the kept count, writes
 * them (nothing, and NULL outputs allowed, when kept is 0).  At most
 * 2^32 - 2 entries in all. */
#define GSA_SUM_NEGATE 4
size_t gsa_coo_sum_workspace_size(int dtype, int64_t m, int64_t n, int64_t total);
int gsa_coo_sum_count(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz_a,
                      const void *rowind_a, const void *colind_a, const void *nzval_a, int op_a, int64_t nnz_b,
                      const void *rowind_b, const void *colind_b, const void *nzval_b, int op_b, int64_t n_diag,
                      const void *lambda, int base, void *workspace, size_t workspace_bytes, int64_t *kept);
int gsa_coo_sum_copy(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t total, int64_t kept,
                     int base, const void *workspace, void *rowind_out, void *colind_out, void *nzval_out);

/* Sums of compressed matrices of one format -- Base.:+ for two GenericSparseMatrixCSR
 * (src/matrix_csr/matrix_csr.jl:290-356, kernels kernel_count_nnz_per_row_csr! /
 * kernel_merge_csr! at src/matrix_csr/matrix_csr_kernels.jl:146-248) or two
 * GenericSparseMatrixCSC (src/matrix_csc/matrix_csc.jl:292-357), and A + λI
 * (src/matrix_csr/matrix_csr.jl:358-402, kernels kernel_count_diag_entries_csr! /
 * kernel_add_uniformscaling_csr! at src/matrix_csr/matrix_csr_kernels.jl:446-507; CSC alike).
 * Per outer entry (row of CSR, column of CSC) the reference's sequential walk: for A + B a
 * two-pointer merge of the stored entries in storage order, equal indices summed a + b (the
 * reference then drops zeros: gsa_dropzeros_* on the result); for A + λI (ptr_b = idx_b = NULL)
 * one more entry where no diagonal is stored, λ added to every stored diagonal and inserted
 * before the first larger index.  Two calls on ONE workspace of
 * gsa_compressed_add_workspace_size(outer_n) bytes: _count returns the result's entry count
 * (synchronizing the stream to read it) and then writes its pointer array ptr_c (outer_n + 1,
 * same base) on the stream; _copy writes idx_c / val_c.  At most 2^32 - 2 entries in A and B
 * together; with Int32 indices at most 2^31 - 1 - base in the result (GSA_ERR_UNSUPPORTED, and
 * ptr_c untouched, beyond either).  negate_b: B's values negated (A - B = A + (-B)).  lambda: host pointer
 * to one value of the dtype (A + λI only). */
size_t gsa_compressed_add_workspace_size(int64_t outer_n);
int gsa_compressed_add_count(void *stream, int itype, int64_t outer_n, const void *ptr_a, const void *idx_a,
                             const void *ptr_b, const void *idx_b, int base, void *workspace, size_t workspace_bytes,
                             void *ptr_c, int64_t *nnz_c);
int gsa_compressed_add_copy(void *stream, int dtype, int itype, int64_t outer_n, const void *ptr_a, const void *idx_a,
                            const void *val_a, const void *ptr_b, const void *idx_b, const void *val_b, int negate_b,
                            const void *lambda, int base, const void *workspace, void *idx_c, void *val_c);

/* Sparse x sparse product C = A * B (SpGEMM) -- Base.:* for two GenericSparseMatrixCSR
 * (src/matrix_csr/matrix_csr.jl:498-556, kernels kernel_count_nnz_spgemm_csr! /
 * kernel_spgemm_csr! at src/matrix_csr/matrix_csr_kernels.jl:250-343) or two
 * GenericSparseMatrixCSC (src/matrix_csc/matrix_csc.jl:500-560, kernels at
 * src/matrix_csc/matrix_csc_kernels.jl:255-345).  A is m x k, B is k x n, both in `format`
 * (0 CSR: ptr = rowptr, idx = colval; 1 CSC: ptr = colptr, idx = rowval) with the same
 * dtype and itype.  C has the same format; every position that a product reaches is stored
 * (zero sums included), indices increasing within each outer entry, and each entry is the
 * sum from zero, in the reference's order, of Julia-rounded products (the reference's bits).
 * _create runs the symbolic phase: it returns the entry count in *nnz_c (synchronizing the
 * stream to read it) and then writes C's pointer array ptr_c (m + 1 for CSR, n + 1 for CSC)
 * on the stream; the handle keeps device scratch and refers to A's and B's arrays, which must
 * stay unchanged until _compute.  _compute writes idx_c / val_c (nnz_c each).  _destroy frees
 * the handle.  At most 2^32 - 2 products (stored A entries times the lengths of the B rows
 * they select); with Int32 indices at most 2^31 - 1 - base entries (GSA_ERR_UNSUPPORTED, and
 * ptr_c untouched, beyond that). */
typedef struct gsa_spgemm gsa_spgemm;
int gsa_spgemm_create(void *stream, int format, int dtype, int itype, int64_t m, int64_t k, int64_t n,
                      const void *ptr_a, const void *idx_a, const void *val_a, int64_t nnz_a, const void *ptr_b,
                      const void *idx_b, const void *val_b, int64_t nnz_b, int base, void *ptr_c, int64_t *nnz_c,
                      gsa_spgemm **handle);
int gsa_spgemm_compute(void *stream, gsa_spgemm *handle, void *idx_c, void *val_c);
int gsa_spgemm_destroy(gsa_spgemm *handle);

/* y = beta*y + alpha*A*x for a CSR matrix and vectors x (n) and y (m), like
 * gsa_csr_mul with opA = opB = N and k = 1, but allocating nothing: no
 * cudaMalloc, no stream-ordered pool, no workspace argument.  No counterpart in
 * the reference.  It is for callers that cannot allocate device memory when they
 * need the product -- a process whose device memory is owned by another pool,
 * or code that must not let an allocation synchronize the device or (in Julia)
 * run the garbage collector.  The kernel's carry slots live in a static device
 * array of 8192 slots (192 KiB, held on every GPU that loads the library until
 * the process exits); a call that would need more slots returns
 * GSA_ERR_INVALID_ARG.  The first call on a device looks up the array's device
 * address, and under CUDA's default lazy module loading it is also the call that
 * loads the library's code and the array onto that device -- which takes device
 * memory.  So make the first call on each device at set-up, while device memory is
 * still free and before any stream capture (or run with CUDA_MODULE_LOADING=EAGER);
 * later calls take no device memory.  All calls share the array: calls that overlap
 * on the GPU race on it.  It runs the pipelined merge-path kernel (GSA_ALGO_PIPE),
 * about three times slower than gsa_csr_mul's default row blocks on the 2048^2
 * Laplacian: it is the entry for callers that cannot allocate, not the fast one.
 * Same tolerance and determinism as gsa_csr_mul. */
int gsa_csr_spmv_noalloc(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                         const void *rowptr, const void *colval, const void *nzval, int base,
                         const void *x, void *y, const void *alpha, const void *beta);

/* ---- plans ----------------------------------------------------------------
 * A plan records which outer entries of one compressed structure (rows of a CSR
 * pointer array, columns of a CSC one) hold more than 32 stored entries, cut into
 * chunks of 512 entries.  With a plan, the row gather (CSR opA = N, CSC opA = T/C)
 * gives each chunk a warp of its own (a long entry is summed chunk by chunk across
 * the whole GPU) and keeps such entries out of the warps of short ones -- what
 * power-law row lengths need; without such entries a plan changes nothing.
 * Creating one copies the pointer array to the host once and synchronizes the
 * stream; the plan holds one device allocation until destroyed.  The structure
 * must not change while its plan is in use.  No counterpart in the reference (its
 * kernels take one work item per row). */
typedef struct gsa_plan gsa_plan;
int gsa_plan_create(void *stream, int itype, int64_t outer_n, int64_t nnz, const void *ptr,
                    int base, gsa_plan **out);
int gsa_plan_destroy(gsa_plan *plan);
/* Longest outer entry, number of planned (longer than 32) entries and of their chunks. */
int gsa_plan_info(const gsa_plan *plan, int64_t *max_len, int64_t *nlong, int64_t *nchunks);
/* Workspace bytes of a planned call with k right-hand sides (0 without planned entries). */
size_t gsa_plan_workspace_size(const gsa_plan *plan, int dtype, int64_t k);

/* gsa_csr_mul / gsa_csc_mul with a plan of the same structure (replace the same
 * reference methods).  The plan applies to both directions under GSA_ALGO_AUTO: the
 * gather (CSR opA = N, CSC opA = T/C) and the outer-block scatter (CSR opA = T/C,
 * CSC opA = N) give planned entries warps of their own.  NULL plan = plain call. */
int gsa_csr_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *rowptr, const void *colval, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes);
int gsa_csc_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *colptr, const void *rowval, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes);

/* COO plans: when the row indices of a COO structure are non-decreasing and within
 * [base, base + m), gsa_coo_plan_create builds its row pointers on the GPU (once; the
 * stream is synchronized) together with an ordinary plan of them, and gsa_coo_mul_planned
 * then runs the CSR kernels on (row pointers, colind, nzval) -- the gather for opA = N,
 * the outer-block scatter for T/C -- instead of the COO kernel.  Otherwise the plan only
 * records that the COO kernel keeps the structure (gsa_coo_plan_info: row_sorted = 0).
 * Replaces the same reference methods as gsa_coo_mul. */
int gsa_coo_plan_create(void *stream, int itype, int64_t m, int64_t n, int64_t nnz, const void *rowind,
                        int base, gsa_plan **out);
int gsa_coo_plan_info(const gsa_plan *plan, int *row_sorted);
int gsa_coo_mul_planned(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                        const void *rowind, const void *colind, const void *nzval, int base, int opA,
                        int64_t k, const void *B, int64_t ldb, int opB, void *C, int64_t ldc,
                        const void *alpha, const void *beta, const gsa_plan *plan, void *workspace,
                        size_t workspace_bytes);

/* ---- three-argument dot ---------------------------------------------------
 * *result = dot(x, op(A), y) = sum over stored entries of conj(x_l) * a * y_r (l = row,
 * r = col for opA = N, swapped for T/C, a conjugated for C); x has rows(op(A)) entries,
 * y cols(op(A)).  result is a HOST pointer to one value of dtype; the call synchronizes
 * the stream (the reference returns the scalar to the host too).  The sum is taken in a
 * fixed order (deterministic).  Replace LinearAlgebra.dot methods generated at
 * src/matrix_csr/matrix_csr.jl:213-277, src/matrix_csc/matrix_csc.jl:219 and
 * src/matrix_coo/matrix_coo.jl:227 (kernels kernel_workgroup_dot_*_N! / _T!).  plan:
 * optional (NULL): a plan of the compressed structure for long outer entries, or for
 * gsa_coo_dot a COO plan (a row-sorted COO then takes the CSR path).
 * workspace: NULL (stream-ordered allocation) or gsa_dot_workspace_size bytes. */
int gsa_csr_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowptr, const void *colval, const void *nzval, int base, int opA,
                const void *x, const void *y, void *result, const gsa_plan *plan,
                void *workspace, size_t workspace_bytes);
int gsa_csc_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *colptr, const void *rowval, const void *nzval, int base, int opA,
                const void *x, const void *y, void *result, const gsa_plan *plan,
                void *workspace, size_t workspace_bytes);
int gsa_coo_dot(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                const void *rowind, const void *colind, const void *nzval, int base, int opA,
                const void *x, const void *y, void *result, const gsa_plan *plan,
                void *workspace, size_t workspace_bytes);
/* format: 0 CSR, 1 CSC, 2 COO (plan: a COO plan, or NULL). */
size_t gsa_dot_workspace_size(int format, int dtype, int itype, int64_t m, int64_t n,
                              const gsa_plan *plan);

/* Workspace bytes for gsa_csr_mul / gsa_csc_mul with these sizes (format:
 * 0 CSR, 1 CSC).  0 means none is needed. */
size_t gsa_mul_workspace_size(int format, int dtype, int itype, int64_t m, int64_t n,
                              int64_t nnz, int opA, int64_t k, int algo);

/* ---- grouped products -------------------------------------------------------
 * Many CSR products C_i = beta_i*C_i + alpha_i*A_i*B_i (A_i m x n with nnz entries,
 * B_i n x k with leading dimension ldb, C_i m x k column-major with ldc) in ONE
 * persistent launch that walks (item, row block or bin-order warps, column group)
 * tiles -- instead of one launch per product, which is what dominates the time of
 * thousands of small products.  alpha/beta hold the bytes of one value of the call's
 * dtype (a double, or re then im).  No counterpart in the reference (one KA launch per
 * mul!). */
typedef struct {
    const void *rowptr, *colval, *nzval;
    const void *B;
    void *C;                   /* m x k, column-major, leading dimension ldc */
    int64_t m, n, nnz, ldb, ldc;
    int32_t k;                 /* right-hand sides */
    int32_t b_rowmajor;        /* 0: B(i, c) at B[i + c*ldb] (ldb >= n); 1: at B[i*ldb + c]
                                  (ldb >= k) -- one entry's k values then share cache lines */
    int64_t first_tile;        /* filled by gsa_grouped_tiles */
    const void *bin_order;     /* NULL (natural row blocks) or gsa_plan_bin_order's view of a
                                  plan of this item's structure */
    int64_t bin_warps;         /* its warp count (0 with a NULL bin_order) */
    unsigned char alpha[16];
    unsigned char beta[16];
} gsa_group_item;              /* 144 bytes */

/* The device view of a plan's bin order for grouped items (NULL and 0 when the plan has no
 * bin order, or has rows of more than 512 entries). */
int gsa_plan_bin_order(const gsa_plan *plan, const void **view, int64_t *warps);

/* Checks the items (host memory), fills first_tile and returns the tile count.
 * columns: right-hand-side columns a thread accumulates (0 = by dtype, 1, 2, 4, 8);
 * the launch must use the same value. */
int gsa_grouped_tiles(int dtype, gsa_group_item *items, int64_t count, int columns, int64_t *ntiles);

/* One grouped launch over a DEVICE array of items prepared by gsa_grouped_tiles.
 * g1_avg: a warp sums one row per thread while its rows average at most g1_avg
 * entries and doubles the lanes per row for every doubling beyond (0 = 6). */
int gsa_grouped_mul(void *stream, int dtype, int itype, int base, const gsa_group_item *d_items,
                    int64_t count, int64_t ntiles, int columns, int g1_avg);

/* A batch: the items copied to the device once (one allocation, synchronizes the
 * stream), run many times with new contents of the same B and C buffers. */
typedef struct gsa_batch gsa_batch;
typedef enum {
    GSA_BATCH_GROUPED = 0,   /* one grouped launch */
    GSA_BATCH_GRAPH = 1,     /* the grouped launch captured into a CUDA graph on first use,
                                replayed afterwards */
    GSA_BATCH_PER_CALL = 2   /* one gsa_csr_mul per item (the per-call baseline) */
} gsa_batch_mode;
int gsa_batch_create(void *stream, int dtype, int itype, int base, const gsa_group_item *items,
                     int64_t count, int columns, int g1_avg, gsa_batch **out);
int gsa_batch_run(gsa_batch *batch, void *stream, int mode);
int gsa_batch_destroy(gsa_batch *batch);

/* ---- format conversions ---------------------------------------------------- */

/* GenericSparseMatrixCSR(::GenericSparseMatrixCOO), src/conversions/conversions.jl:282-323
 * (keys src/conversions/conversion_kernels.jl:49-57): stable sort of the triplets by
 * (row, col) -- duplicates kept in input order -- then rowptr (m+1 entries,
 * rowptr[m] == nnz + base).  Outputs must not overlap inputs. */
int gsa_coo_to_csr(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowind, const void *colind, const void *nzval, int base,
                   void *rowptr_out, void *colval_out, void *nzval_out, void *workspace,
                   size_t workspace_bytes);

/* GenericSparseMatrixCSC(::GenericSparseMatrixCOO), src/conversions/conversions.jl:171-212
 * (keys src/conversions/conversion_kernels.jl:38-46): the same with (col, row) order. */
int gsa_coo_to_csc(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowind, const void *colind, const void *nzval, int base,
                   void *colptr_out, void *rowval_out, void *nzval_out, void *workspace,
                   size_t workspace_bytes);

/* Workspace bytes for gsa_coo_to_csr (colmajor == 0) / gsa_coo_to_csc (1). */
size_t gsa_coo_to_compressed_workspace_size(int colmajor, int dtype, int itype, int64_t m,
                                            int64_t n, int64_t nnz);

/* GenericSparseMatrixCOO(::GenericSparseMatrixCSR), src/conversions/conversions.jl:264-280
 * (kernel_csr_to_coo!, src/conversions/conversion_kernels.jl:20-35). */
int gsa_csr_to_coo(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *rowptr, const void *colval, const void *nzval, int base,
                   void *rowind_out, void *colind_out, void *nzval_out);

/* GenericSparseMatrixCOO(::GenericSparseMatrixCSC), src/conversions/conversions.jl:153-169
 * (kernel_csc_to_coo!, src/conversions/conversion_kernels.jl:2-17). */
int gsa_csc_to_coo(void *stream, int dtype, int itype, int64_t m, int64_t n, int64_t nnz,
                   const void *colptr, const void *rowval, const void *nzval, int base,
                   void *rowind_out, void *colind_out, void *nzval_out);

/* Synchronizes the stream, then reads and clears the device error word that
 * bounded device-side waits set when they give up (no counterpart in the
 * reference).  GSA_OK, or GSA_ERR_TIMEOUT if any wait gave up since the last
 * check; the results of the call that timed out are not valid. */
int gsa_check_device_status(void *stream);

/* ---- structure check ------------------------------------------------------
 * The reference constructors skip the structural check
 * (src/matrix_csr/matrix_csr.jl:49, "TODO: this uses scalar indexing").
 * This one runs on the device and synchronizes the stream: ptr[0] == base,
 * ptr non-decreasing, ptr[outer_n] == nnz + base and every index in
 * [base, inner_n + base).  Returns GSA_OK or GSA_ERR_STRUCTURE. */
int gsa_validate_compressed(void *stream, int itype, int64_t outer_n, int64_t inner_n,
                            int64_t nnz, const void *ptr, const void *idx, int base);

#ifdef __cplusplus
}
#endif

#endif /* GSA_H */
