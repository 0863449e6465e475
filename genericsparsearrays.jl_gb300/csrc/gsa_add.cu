// Sparse + dense: C += A for a dense column-major C -- the kernel of `A + B` with a dense B
// (src/core.jl:66-88: C = copy(B), then _add_sparse_to_dense!, whose kernels are
// kernel_add_sparse_to_dense_{csr,csc,coo}! at src/matrix_csr/matrix_csr_kernels.jl:133-145
// and the CSC/COO counterparts).  The reference gives each row (column, entry) one work
// item; here a warp owns 32 outer entries with G lanes each (as the row gather), and every
// entry is added with an atomic, so duplicate (row, col) entries -- in one outer entry or
// in a COO -- add up whatever lane holds them.
#include "gsa_rows.cuh"

namespace gsa {

template <typename V, typename I, int G>
__device__ __forceinline__ void add_rows(const CompressedArgs<V, I> &a, bool csr, V *C, int64_t ldc,
                                         int64_t row0, Off<I> b, Off<I> e) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    constexpr int RPP = 32 / G;
    const O inner = sizeof(O) == 8 ? (O)a.inner_n
                                   : (O)(a.inner_n < 0xffffffffLL ? a.inner_n : 0xffffffffLL);
    const O base = (O)a.base;
#pragma unroll 1
    for (int p = 0; p < G; ++p) {
        const int q = p * RPP + lane / G;
        const O qb = G == 1 ? b : (O)__shfl_sync(0xffffffffu, b, q);
        const O qe = G == 1 ? e : (O)__shfl_sync(0xffffffffu, e, q);
        const int64_t o = row0 + q;
        for (O j = qb + (O)(lane % G); j < qe; j += G) {
            const O ii = (O)ld_stream(a.idx + j) - base;
            const V v = ld_stream(a.val + j);
            if (ii >= inner) continue;
            const int64_t r = csr ? o : (int64_t)ii, c = csr ? (int64_t)ii : o;
            atomic_add(C + r + c * ldc, v);
        }
    }
}

template <typename V, typename I>
__global__ void __launch_bounds__(RB_THREADS)
add_compressed_kernel(CompressedArgs<V, I> a, bool csr, V *C, int64_t ldc) {
    const int64_t row0 = (int64_t)blockIdx.x * RB_THREADS + (threadIdx.x & ~31);
    Off<I> b, e;
    int skip;
    const int64_t avg = warp_extent(a, row0, nullptr, b, e, skip);
    dispatch_lanes(avg, G1_AVG, [&](auto g) { add_rows<V, I, decltype(g)::value>(a, csr, C, ldc, row0, b, e); });
}

template <typename V, typename I>
__global__ void __launch_bounds__(256)
add_coo_kernel(int64_t nnz, const I *__restrict__ rowind, const I *__restrict__ colind,
               const V *__restrict__ val, int base, int64_t m, int64_t n, V *C, int64_t ldc) {
    for (int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * 256) {
        const int64_t r = (int64_t)ld_stream(rowind + e) - base, c = (int64_t)ld_stream(colind + e) - base;
        if ((uint64_t)r >= (uint64_t)m || (uint64_t)c >= (uint64_t)n) continue;
        atomic_add(C + r + c * ldc, ld_stream(val + e));
    }
}

template <typename V, typename I>
int launch_add_to_dense(cudaStream_t s, int fmt, int64_t m, int64_t n, int64_t nnz, const I *p0, const I *p1,
                        const V *val, int base, V *C, int64_t ldc) {
    if (m == 0 || n == 0 || nnz == 0) return GSA_OK;
    timer_before(s);
    if (fmt == 2) {
        int64_t blocks = ceil_div(nnz, 256);
        if (blocks > 152 * 32) blocks = 152 * 32;
        add_coo_kernel<V, I><<<(unsigned)blocks, 256, 0, s>>>(nnz, p0, p1, val, base, m, n, C, ldc);
    } else {
        const bool csr = fmt == 0;
        CompressedArgs<V, I> a;
        a.outer_n = csr ? m : n;
        a.inner_n = csr ? n : m;
        a.nnz = nnz;
        a.ptr = p0;
        a.idx = p1;
        a.val = val;
        a.base = base;
        a.conjA = false;
        const int64_t blocks = ceil_div(a.outer_n, RB_THREADS);
        if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many outer entries");
        add_compressed_kernel<V, I><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, csr, C, ldc);
    }
    timer_after(s);
    return check_cuda(cudaGetLastError(), "add_to_dense");
}

#define GSA_INST_ADD(V, I)                                                                         \
    template int launch_add_to_dense<V, I>(cudaStream_t, int, int64_t, int64_t, int64_t, const I *, \
                                           const I *, const V *, int, V *, int64_t);
GSA_INST_ADD(float, int32_t)
GSA_INST_ADD(float, int64_t)
GSA_INST_ADD(double, int32_t)
GSA_INST_ADD(double, int64_t)
GSA_INST_ADD(cf32, int32_t)
GSA_INST_ADD(cf32, int64_t)
GSA_INST_ADD(cf64, int32_t)
GSA_INST_ADD(cf64, int64_t)
GSA_INST_ADD(int32_t, int32_t)
GSA_INST_ADD(int32_t, int64_t)
GSA_INST_ADD(int64_t, int32_t)
GSA_INST_ADD(int64_t, int64_t)

}  // namespace gsa
