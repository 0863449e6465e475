// Sums of compressed matrices: A + B for two CSR (or two CSC) matrices and A + λI.
//
// A + B follows kernel_count_nnz_per_row_csr! / kernel_merge_csr!
// (src/matrix_csr/matrix_csr_kernels.jl:146-248, the CSC kernels at
// src/matrix_csc/matrix_csc_kernels.jl:146-250): per outer entry a two-pointer walk over A's
// and B's stored entries in storage order -- the smaller index first, equal indices summed
// a + b.  The walk is kept as it is (a thread per outer entry, counting pass, scan, writing
// pass), so rows that are unsorted or hold repeated indices give the reference's result too;
// the caller then drops zeros (the reference returns dropzeros(C)).
// A + λI follows kernel_count_diag_entries_csr! / kernel_add_uniformscaling_csr!
// (src/matrix_csr/matrix_csr_kernels.jl:446-507): an outer entry without a stored diagonal gets
// one more entry; λ is added to every stored diagonal and inserted before the first entry past
// the diagonal, or at the end.  Writes stay inside each entry's counted room.
#include <type_traits>

#include "gsa_internal.cuh"

namespace gsa {
namespace {

template <typename V> __device__ __forceinline__ V negated(V a) {  // integers wrap, as in Julia
    using U = typename std::make_unsigned<V>::type;
    return (V)(U(0) - (U)a);
}
template <> __device__ __forceinline__ float negated(float a) { return flip_sign_if(a, true); }
template <> __device__ __forceinline__ double negated(double a) { return flip_sign_if(a, true); }
template <> __device__ __forceinline__ cf32 negated(cf32 a) { return cf32{flip_sign_if(a.re, true), flip_sign_if(a.im, true)}; }
template <> __device__ __forceinline__ cf64 negated(cf64 a) { return cf64{flip_sign_if(a.re, true), flip_sign_if(a.im, true)}; }

// cnt[o] = entries of the merged outer entry o; cnt[outer_n] = 0.
template <typename I>
__global__ void merge_count_kernel(int64_t outer_n, const I *__restrict__ pa, const I *__restrict__ ia,
                                   const I *__restrict__ pb, const I *__restrict__ ib, int base,
                                   uint32_t *__restrict__ cnt) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o <= outer_n; o += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        if (o < outer_n) {
            int64_t a = (int64_t)__ldg(pa + o) - base, ae = (int64_t)__ldg(pa + o + 1) - base;
            int64_t b = (int64_t)__ldg(pb + o) - base, be = (int64_t)__ldg(pb + o + 1) - base;
            while (a < ae && b < be) {
                const I x = __ldg(ia + a), y = __ldg(ib + b);
                if (x < y) ++a;
                else if (x > y) ++b;
                else { ++a; ++b; }
                ++c;
            }
            c += (uint32_t)((ae > a ? ae - a : 0) + (be > b ? be - b : 0));
        }
        cnt[o] = c;
    }
}

template <typename V, typename I>
__global__ void merge_fill_kernel(int64_t outer_n, const I *__restrict__ pa, const I *__restrict__ ia,
                                  const V *__restrict__ va, const I *__restrict__ pb, const I *__restrict__ ib,
                                  const V *__restrict__ vb, bool neg_b, int base, const uint32_t *__restrict__ cptr,
                                  I *__restrict__ idx_out, V *__restrict__ val_out) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < outer_n; o += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = (int64_t)__ldg(pa + o) - base, ae = (int64_t)__ldg(pa + o + 1) - base;
        int64_t b = (int64_t)__ldg(pb + o) - base, be = (int64_t)__ldg(pb + o + 1) - base;
        uint32_t w = cptr[o];
        const uint32_t end = cptr[o + 1];
        while ((a < ae || b < be) && w < end) {
            if (a < ae && b < be) {
                const I x = __ldg(ia + a), y = __ldg(ib + b);
                if (x < y) {
                    idx_out[w] = x;
                    val_out[w] = ldg(va + a++);
                } else if (x > y) {
                    const V v = ldg(vb + b++);
                    idx_out[w] = y;
                    val_out[w] = neg_b ? negated(v) : v;
                } else {
                    const V v = ldg(vb + b++);
                    idx_out[w] = x;
                    val_out[w] = add(ldg(va + a++), neg_b ? negated(v) : v);
                }
            } else if (a < ae) {
                idx_out[w] = __ldg(ia + a);
                val_out[w] = ldg(va + a++);
            } else {
                const V v = ldg(vb + b);
                idx_out[w] = __ldg(ib + b++);
                val_out[w] = neg_b ? negated(v) : v;
            }
            ++w;
        }
    }
}

template <typename I>
__global__ void diag_count_kernel(int64_t n, const I *__restrict__ pa, const I *__restrict__ ia, int base,
                                  uint32_t *__restrict__ cnt) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o <= n; o += (int64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        if (o < n) {
            const int64_t b = (int64_t)__ldg(pa + o) - base, e = (int64_t)__ldg(pa + o + 1) - base;
            bool found = false;
            for (int64_t j = b; j < e && !found; ++j) found = (int64_t)__ldg(ia + j) - base == o;
            c = (uint32_t)(e - b) + (found ? 0u : 1u);
        }
        cnt[o] = c;
    }
}

template <typename V, typename I>
__global__ void diag_fill_kernel(int64_t n, const I *__restrict__ pa, const I *__restrict__ ia,
                                 const V *__restrict__ va, V lam, int base, const uint32_t *__restrict__ cptr,
                                 I *__restrict__ idx_out, V *__restrict__ val_out) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = (int64_t)__ldg(pa + o) - base, e = (int64_t)__ldg(pa + o + 1) - base;
        uint32_t w = cptr[o];
        const uint32_t end = cptr[o + 1];
        bool written = false;
        for (int64_t j = b; j < e; ++j) {
            const I ij = __ldg(ia + j);
            const int64_t col = (int64_t)ij - base;
            if (!written && col > o) {
                if (w < end) {
                    idx_out[w] = (I)(o + base);
                    val_out[w] = lam;
                }
                ++w;
                written = true;
            }
            if (w < end) {
                idx_out[w] = ij;
                if (col == o) {
                    val_out[w] = add(ldg(va + j), lam);
                    written = true;
                } else {
                    val_out[w] = ldg(va + j);
                }
            }
            ++w;
        }
        if (!written && w < end) {
            idx_out[w] = (I)(o + base);
            val_out[w] = lam;
        }
    }
}

template <typename I>
__global__ void merged_pointers_kernel(int64_t outer_n, const uint32_t *__restrict__ cptr, int base,
                                       I *__restrict__ ptr_out) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o <= outer_n; o += (int64_t)gridDim.x * blockDim.x)
        ptr_out[o] = (I)((int64_t)cptr[o] + base);
}

unsigned mg_grid(int64_t n) {
    int64_t b = ceil_div(n, 256);
    if (b > 152 * 32) b = 152 * 32;
    return (unsigned)(b > 0 ? b : 1);
}

struct MergeLayout {
    size_t cnt, cptr, bsums, bytes;
};
MergeLayout merge_layout(int64_t outer_n) {
    MergeLayout L;
    Carver cv(nullptr);
    L.cnt = cv.reserve<uint32_t>(outer_n + 1);
    L.cptr = cv.reserve<uint32_t>(outer_n + 1);
    L.bsums = cv.reserve<uint32_t>(scan_block_sums(outer_n + 1));
    L.bytes = align_up(cv.off, 256);
    return L;
}

// Counting pass, scan, pointer array, and the count on the host.
// The stored entry count of a compressed operand: its last pointer minus base (0 if smaller).
int64_t stored_count(int itype, int64_t last, int base) {
    const int64_t v = (itype == GSA_IDX32 ? (int64_t)(int32_t)last : last) - base;
    return v > 0 ? v : 0;
}

// Scans the per-outer-entry counts, checks that the total fits (the scan is 32-bit, and Int32
// pointers hold at most 2^31 - 1), then writes the result's pointers.  ptr_b NULL: A + λI,
// at most one entry more per outer entry.
int finish_count(cudaStream_t s, int64_t outer_n, void *ws, int itype, int base, const void *ptr_a,
                 const void *ptr_b, void *ptr_c, int64_t *nnz_c) {
    const MergeLayout L = merge_layout(outer_n);
    char *w = (char *)ws;
    uint32_t *cnt = (uint32_t *)(w + L.cnt), *cptr = (uint32_t *)(w + L.cptr);
    int rc = scan_u32(s, cnt, cptr, outer_n + 1, (uint32_t *)(w + L.bsums));
    if (rc) return rc;
    const size_t is = itype == GSA_IDX32 ? 4 : 8;
    uint32_t total = 0;
    int64_t last_a = 0, last_b = 0;  // the low `is` bytes are the pointer (little-endian)
    rc = check_cuda(cudaMemcpyAsync(&total, cptr + outer_n, sizeof(total), cudaMemcpyDeviceToHost, s), "sum: count");
    if (!rc) rc = check_cuda(cudaMemcpyAsync(&last_a, (const char *)ptr_a + outer_n * is, is, cudaMemcpyDeviceToHost, s),
                             "sum: nnz of A");
    if (!rc && ptr_b)
        rc = check_cuda(cudaMemcpyAsync(&last_b, (const char *)ptr_b + outer_n * is, is, cudaMemcpyDeviceToHost, s),
                        "sum: nnz of B");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "sum: sync");
    if (rc) return rc;
    const int64_t bound = stored_count(itype, last_a, base) + (ptr_b ? stored_count(itype, last_b, base) : outer_n);
    if (bound >= 0xffffffffLL)
        return fail(GSA_ERR_UNSUPPORTED, "a sum of up to %lld entries; at most 2^32 - 2 are supported", (long long)bound);
    if (itype == GSA_IDX32 && (int64_t)total + base > 0x7fffffffLL)
        return fail(GSA_ERR_UNSUPPORTED, "the sum has %u entries, more than Int32 pointers can address", total);
    if (itype == GSA_IDX32) merged_pointers_kernel<int32_t><<<mg_grid(outer_n + 1), 256, 0, s>>>(outer_n, cptr, base, (int32_t *)ptr_c);
    else merged_pointers_kernel<int64_t><<<mg_grid(outer_n + 1), 256, 0, s>>>(outer_n, cptr, base, (int64_t *)ptr_c);
    rc = check_cuda(cudaGetLastError(), "merged_pointers_kernel");
    if (!rc) *nnz_c = total;
    return rc;
}

struct MergeCountBody {
    cudaStream_t s; int64_t outer_n; const void *pa, *ia, *pb, *ib; int base; void *ws;
    template <typename V, typename I> int operator()() {
        const MergeLayout L = merge_layout(outer_n);
        uint32_t *cnt = (uint32_t *)((char *)ws + L.cnt);
        if (pb) merge_count_kernel<I><<<mg_grid(outer_n + 1), 256, 0, s>>>(outer_n, (const I *)pa, (const I *)ia,
                                                                            (const I *)pb, (const I *)ib, base, cnt);
        else diag_count_kernel<I><<<mg_grid(outer_n + 1), 256, 0, s>>>(outer_n, (const I *)pa, (const I *)ia, base, cnt);
        return check_cuda(cudaGetLastError(), "sum: count kernel");
    }
};

struct MergeFillBody {
    cudaStream_t s; int64_t outer_n; const void *pa, *ia, *va, *pb, *ib, *vb; bool neg_b; const void *lam; int base;
    const void *ws; void *idx_c, *val_c;
    template <typename V, typename I> int operator()() {
        const MergeLayout L = merge_layout(outer_n);
        const uint32_t *cptr = (const uint32_t *)((const char *)ws + L.cptr);
        if (pb)
            merge_fill_kernel<V, I><<<mg_grid(outer_n), 256, 0, s>>>(outer_n, (const I *)pa, (const I *)ia, (const V *)va,
                                                                     (const I *)pb, (const I *)ib, (const V *)vb, neg_b,
                                                                     base, cptr, (I *)idx_c, (V *)val_c);
        else
            diag_fill_kernel<V, I><<<mg_grid(outer_n), 256, 0, s>>>(outer_n, (const I *)pa, (const I *)ia, (const V *)va,
                                                                    *(const V *)lam, base, cptr, (I *)idx_c, (V *)val_c);
        return check_cuda(cudaGetLastError(), "sum: fill kernel");
    }
};

bool mg_misaligned(const void *p, size_t a) { return a && ((uintptr_t)p % a) != 0; }

}  // namespace
}  // namespace gsa

extern "C" {

size_t gsa_compressed_add_workspace_size(int64_t outer_n) {
    return outer_n < 0 ? 0 : gsa::merge_layout(outer_n).bytes;
}

int gsa_compressed_add_count(void *stream, int itype, int64_t outer_n, const void *ptr_a, const void *idx_a,
                             const void *ptr_b, const void *idx_b, int base, void *workspace, size_t workspace_bytes,
                             void *ptr_c, int64_t *nnz_c) {
    using namespace gsa;
    const size_t is = itype_size(itype);
    if (!is) return fail(GSA_ERR_UNSUPPORTED, "unsupported itype %d", itype);
    if (outer_n < 0 || outer_n >= 0xfffffffeLL) return fail(GSA_ERR_INVALID_ARG, "outer size out of range");
    if (!ptr_a || !ptr_c || !nnz_c || !workspace) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (workspace_bytes < merge_layout(outer_n).bytes) return fail(GSA_ERR_INVALID_ARG, "workspace too small");
    if (mg_misaligned(ptr_a, is) || mg_misaligned(idx_a, is) || mg_misaligned(ptr_b, is) || mg_misaligned(idx_b, is) ||
        mg_misaligned(ptr_c, is))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    MergeCountBody body{(cudaStream_t)stream, outer_n, ptr_a, idx_a, ptr_b, idx_b, base, workspace};
    int rc = dispatch_vi(GSA_F64, itype, body);
    if (!rc) rc = finish_count((cudaStream_t)stream, outer_n, workspace, itype, base, ptr_a, ptr_b, ptr_c, nnz_c);
    return rc;
}

int gsa_compressed_add_copy(void *stream, int dtype, int itype, int64_t outer_n, const void *ptr_a, const void *idx_a,
                            const void *val_a, const void *ptr_b, const void *idx_b, const void *val_b, int negate_b,
                            const void *lambda, int base, const void *workspace, void *idx_c, void *val_c) {
    using namespace gsa;
    const size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (outer_n < 0 || !ptr_a || !workspace) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (!ptr_b && !lambda) return fail(GSA_ERR_INVALID_ARG, "either B or lambda is needed");
    if (mg_misaligned(idx_c, is) || mg_misaligned(val_c, vs) || mg_misaligned(val_a, vs) || mg_misaligned(val_b, vs))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    MergeFillBody body{(cudaStream_t)stream, outer_n, ptr_a, idx_a, val_a, ptr_b, idx_b, val_b, negate_b != 0,
                       lambda, base, workspace, idx_c, val_c};
    return dispatch_vi(dtype, itype, body);
}

}  // extern "C"
