// Three-argument dot(x, op(A), y) = x' op(A) y -- LinearAlgebra.dot for the three
// formats (src/matrix_csr/matrix_csr.jl:213-277 with kernel_workgroup_dot_csr_{N,T}! at
// src/matrix_csr/matrix_csr_kernels.jl:47-131; the CSC and COO methods and kernels at
// src/matrix_csc/matrix_csc.jl:219, src/matrix_csc/matrix_csc_kernels.jl:47-131,
// src/matrix_coo/matrix_coo.jl:227, src/matrix_coo/matrix_coo_kernels.jl:45-130).
// Every stored entry (row, col) contributes conj(x_l) * a * y_r, l = row and r = col for
// op = N (swapped for T/C, a conjugated for C).
//
// The reference gives each work item a stride of rows and sums the items' partials on
// one thread per block, then on the host.  Here the compressed formats reuse the row
// gather's layout: a warp owns 32 outer entries, G lanes per entry from their average
// length (planned long entries get warps of their own, chunk by chunk; ComplexF64 walks
// the plan's bin order, rows grouped by length, as the product does), and sums along
// each entry the vector that pairs with the inner index -- s_o = sum_j a_oj y_j when x
// pairs with the outer index (CSR N, CSC T/C), t_o = sum_j conj(x_j) a_oj when y does
// (CSR T/C, CSC N) -- with one fused multiply-add per entry, then multiplies once per
// entry by conj(x_o) or y_o.  COO gives each warp 32 consecutive entries.  Each warp
// writes one partial to a fixed slot; a second kernel adds the slots in a fixed order,
// so the result does not depend on scheduling.
#include "gsa_rows.cuh"

namespace gsa {

template <typename V> struct DotVecs {
    const V *x, *y;
    bool outer_left;  // x pairs with the outer index
};

template <typename V> __device__ __forceinline__ V conj_v(V v) { return conj_if(v, true); }

// sum over j = jb, jb+S, ... < je of the inner products of one outer entry
template <typename V, typename I, int S, int U>
__device__ __forceinline__ V dot_range(const CompressedArgs<V, I> &a, const DotVecs<V> &d, Off<I> j,
                                       Off<I> je) {
    using O = Off<I>;
    const O inner = sizeof(O) == 8 ? (O)a.inner_n
                                   : (O)(a.inner_n < 0xffffffffLL ? a.inner_n : 0xffffffffLL);
    const O base = (O)a.base;
    V acc = VT<V>::zero();
    if (U > 1) {
        for (; j + (O)((U - 1) * S) < je; j += U * S) {
            O ci[U];
            V av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ci[u] = (O)a.idx[j + u * S] - base;
                av[u] = conj_if(a.val[j + u * S], a.conjA);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = ci[u] < inner;
                if (d.outer_left) acc = mac(acc, av[u], ok ? ldg(d.y + ci[u]) : VT<V>::zero());
                else acc = mac(acc, ok ? conj_v(ldg(d.x + ci[u])) : VT<V>::zero(), av[u]);
            }
        }
    }
    for (; j < je; j += S) {
        const O c1 = (O)a.idx[j] - base;
        const bool ok = c1 < inner;
        const V av = conj_if(a.val[j], a.conjA);
        if (d.outer_left) acc = mac(acc, av, ok ? ldg(d.y + c1) : VT<V>::zero());
        else acc = mac(acc, ok ? conj_v(ldg(d.x + c1)) : VT<V>::zero(), av);
    }
    return acc;
}

template <typename V> __device__ __forceinline__ V outer_term(const DotVecs<V> &d, int64_t o, V s) {
    return d.outer_left ? mul(conj_v(ldg(d.x + o)), s) : mul(s, ldg(d.y + o));
}

// this lane's share of the warp's 32 outer entries, G lanes per entry
template <typename V, typename I, int G>
__device__ __forceinline__ V dot_rows(const CompressedArgs<V, I> &a, const DotVecs<V> &d, int64_t row0,
                                      Off<I> b, Off<I> e, int skip) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    constexpr int RPP = 32 / G;
    V total = VT<V>::zero();
#pragma unroll 1
    for (int p = 0; p < G; ++p) {
        const int q = p * RPP + lane / G;
        const O qb = G == 1 ? b : (O)__shfl_sync(0xffffffffu, b, q);
        const O qe = G == 1 ? e : (O)__shfl_sync(0xffffffffu, e, q);
        const int qskip = G == 1 ? skip : __shfl_sync(0xffffffffu, skip, q);
        V s = dot_range<V, I, G, (G == 1 ? 1 : 2)>(a, d, qb + (O)(lane % G), qe);
        if (G > 1) {
#pragma unroll
            for (int m = G / 2; m > 0; m >>= 1) s = add(s, shfl_xor(s, m, G));
        }
        const int64_t o = row0 + q;
        if (lane % G == 0 && o < a.outer_n && !qskip) total = add(total, outer_term(d, o, s));
    }
    return total;
}

template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = add(v, shfl_xor(v, m));
    return v;
}

template <typename V, typename I>
__global__ void __launch_bounds__(RB_THREADS)
dot_compressed_kernel(CompressedArgs<V, I> a, DotVecs<V> d, int64_t nrb, PlanRows L, V *partial) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const int64_t unit = blockIdx.x;
    const int64_t slot = unit * RB_WARPS + (threadIdx.x >> 5);
    V t = VT<V>::zero();
    if (unit >= nrb) {  // a chunk of a planned long outer entry
        const int64_t chunk = (unit - nrb) * RB_WARPS + (threadIdx.x >> 5);
        if (chunk < L.nchunks) {
            const int sl = L.chunk_slot[chunk];
            const int64_t o = L.row[sl];
            const O nz = (O)a.nnz, base = (O)a.base;
            O rb = (O)__ldg(a.ptr + o) - base;
            O re = (O)__ldg(a.ptr + o + 1) - base;
            rb = rb < nz ? rb : nz;
            re = re < nz ? re : nz;
            const O jb = rb + (O)(chunk - L.first[sl]) * (O)CHUNK;
            const O je = jb < re && re - jb > (O)CHUNK ? jb + (O)CHUNK : re;
            V s = jb < je ? dot_range<V, I, 32, UNROLL>(a, d, jb + (O)lane, je) : VT<V>::zero();
            s = warp_sum(s);
            if (lane == 0) t = outer_term(d, o, s);
        }
    } else {
        const int64_t row0 = unit * RB_THREADS + (threadIdx.x & ~31);
        Off<I> b, e;
        int skip;
        const int64_t avg = warp_extent(a, row0, L.skip_mask, b, e, skip);
        dispatch_lanes(avg, G1_AVG, [&](auto g) { t = dot_rows<V, I, decltype(g)::value>(a, d, row0, b, e, skip); });
    }
    t = warp_sum(t);
    if (lane == 0) partial[slot] = t;
}

// The same over the plan's bin order (rows grouped by length, G lanes each), then the bin
// set's chunks of rows over 512 entries: used where the FP64 pipe binds (ComplexF64).
template <typename V, typename I, int G>
__device__ __forceinline__ V dot_binned_rows(const CompressedArgs<V, I> &a, const DotVecs<V> &d, int64_t pos0,
                                             int64_t pend, const gsa_bin_order &bv) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const int64_t i = pos0 + lane / G;
    const bool valid = i < pend;
    int64_t o = 0;
    O b = 0, e = 0;
    if (valid) o = bin_row(a, bv, i, b, e);
    V s = dot_range<V, I, G, (G == 1 ? 1 : 2)>(a, d, b + (O)(lane % G), e);
    if (G > 1) {
#pragma unroll
        for (int m = G / 2; m > 0; m >>= 1) s = add(s, shfl_xor(s, m, G));
    }
    return (lane % G == 0 && valid && o < a.outer_n) ? outer_term(d, o, s) : VT<V>::zero();
}

template <typename V, typename I>
__global__ void __launch_bounds__(RB_THREADS)
dot_binned_kernel(CompressedArgs<V, I> a, DotVecs<V> d, gsa_bin_order bv, PlanRows L, V *partial) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const int64_t w = (int64_t)blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    V t = VT<V>::zero();
    if (w < bv.nwarps) {
        int64_t pos0, pend;
        int G;
        bin_warp(bv, w, pos0, pend, G);
        dispatch_lanes(G, 1, [&](auto g) { t = dot_binned_rows<V, I, decltype(g)::value>(a, d, pos0, pend, bv); });
    } else if (w - bv.nwarps < L.nchunks) {  // a chunk of a row over 512 entries
        const int64_t chunk = w - bv.nwarps;
        const int sl = L.chunk_slot[chunk];
        const int64_t o = L.row[sl];
        const O nz = (O)a.nnz, base = (O)a.base;
        O rb = (O)__ldg(a.ptr + o) - base;
        O re = (O)__ldg(a.ptr + o + 1) - base;
        rb = rb < nz ? rb : nz;
        re = re < nz ? re : nz;
        const O jb = rb + (O)(chunk - L.first[sl]) * (O)CHUNK;
        const O je = jb < re && re - jb > (O)CHUNK ? jb + (O)CHUNK : re;
        V s = jb < je ? dot_range<V, I, 32, UNROLL>(a, d, jb + (O)lane, je) : VT<V>::zero();
        s = warp_sum(s);
        if (lane == 0) t = outer_term(d, o, s);
    }
    t = warp_sum(t);
    if (lane == 0) partial[w] = t;
}

constexpr int COO_DOT_CTAS = 1216;  // 152 SMs x 8, a fixed grid: the slot order is fixed

template <typename V, typename I>
__global__ void __launch_bounds__(256)
dot_coo_kernel(int64_t nnz, const I *__restrict__ rowind, const I *__restrict__ colind,
               const V *__restrict__ val, int base, bool trans, bool conjA, const V *__restrict__ x,
               const V *__restrict__ y, int64_t m, int64_t n, V *partial) {
    __shared__ V s_warp[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    V acc = VT<V>::zero();
    for (int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * 256) {
        const int64_t r = (int64_t)ld_stream(rowind + e) - base, c = (int64_t)ld_stream(colind + e) - base;
        if ((uint64_t)r >= (uint64_t)m || (uint64_t)c >= (uint64_t)n) continue;  // outside the matrix
        const V av = conj_if(ld_stream(val + e), conjA);
        const int64_t l = trans ? c : r, rr = trans ? r : c;
        acc = mac(acc, mul(conj_v(ldg(x + l)), av), ldg(y + rr));
    }
    acc = warp_sum(acc);
    if (lane == 0) s_warp[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        V t = VT<V>::zero();
        for (int w = 0; w < 8; ++w) t = add(t, s_warp[w]);
        partial[blockIdx.x] = t;
    }
}

// out[0] = sum of partial[0..count) in a fixed order: thread t adds slots t, t + 1024, ...,
// then a fixed tree over the threads.
template <typename V>
__global__ void __launch_bounds__(1024) dot_finish_kernel(const V *__restrict__ partial, int64_t count, V *out) {
    __shared__ V s[1024];
    V t = VT<V>::zero();
    for (int64_t i = threadIdx.x; i < count; i += 1024) t = add(t, partial[i]);
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = add(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = s[0];
}

template <typename V, typename I>
size_t dot_workspace_size(int fmt, int64_t outer_n, const Plan *plan) {
    int64_t slots;
    if (fmt == 2) slots = COO_DOT_CTAS;
    else slots = (ceil_div(outer_n, RB_THREADS) + ceil_div(plan ? plan->nat.nchunks : 0, RB_WARPS)) * RB_WARPS;
    if (fmt != 2 && plan && plan->nbin_warps > 0) {  // room for the bin order too
        const int64_t b = ceil_div(plan->nbin_warps + plan->bin.nchunks, RB_WARPS) * RB_WARPS;
        slots = b > slots ? b : slots;
    }
    return align_up((size_t)(slots + 1) * sizeof(V), 256);
}

// the slots' sum, in a fixed order, to the host
template <typename V>
static int finish_dot(cudaStream_t s, V *partial, int64_t slots, void *result_host) {
    int rc = check_cuda(cudaGetLastError(), "dot kernel");
    if (rc) return rc;
    dot_finish_kernel<V><<<1, 1024, 0, s>>>(partial, slots, partial + slots);
    rc = check_cuda(cudaGetLastError(), "dot_finish_kernel");
    if (!rc) rc = check_cuda(cudaMemcpyAsync(result_host, partial + slots, sizeof(V), cudaMemcpyDeviceToHost, s),
                             "dot: result");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "dot: sync");
    return rc;
}

template <typename V, typename I>
int launch_dot(cudaStream_t s, int fmt, int opA, int64_t m, int64_t n, int64_t nnz, const I *p0,
               const I *p1, const V *val, int base, const V *x, const V *y, const Plan *plan,
               void *ws, size_t ws_bytes, void *result_host) {
    const size_t need = dot_workspace_size<V, I>(fmt, fmt == 0 ? m : n, plan);
    if (ws_bytes < need) return fail(GSA_ERR_INVALID_ARG, "dot workspace too small");
    V *partial = (V *)ws;
    int64_t slots = 0;
    const bool trans = opA != GSA_OP_N, conjA = opA == GSA_OP_C;
    if (fmt == 2) {
        slots = COO_DOT_CTAS;
        timer_before(s);
        dot_coo_kernel<V, I><<<COO_DOT_CTAS, 256, 0, s>>>(nnz, p0, p1, val, base, trans, conjA, x, y, m, n,
                                                          partial);
        timer_after(s);
    } else {
        CompressedArgs<V, I> a;
        const bool csr = fmt == 0;
        a.outer_n = csr ? m : n;
        a.inner_n = csr ? n : m;
        a.nnz = nnz;
        a.ptr = p0;
        a.idx = p1;
        a.val = val;
        a.base = base;
        a.conjA = conjA;
        // CSR N and CSC T/C: x pairs with the outer index
        const DotVecs<V> d{x, y, csr ? !trans : trans};
        if constexpr (std::is_same<V, cf64>::value)  // FP64-bound: bin order (no other instances)
        if (plan && plan->nbin_warps > 0) {
            if (plan->outer_n != a.outer_n || plan->nnz != nnz)
                return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
            const gsa_bin_order bv = plan->order;
            const PlanRows L = plan_rows(plan->bin);
            const int64_t units = ceil_div(plan->nbin_warps + plan->bin.nchunks, RB_WARPS);
            slots = units * RB_WARPS;
            if (units > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many outer entries");
            timer_before(s);
            dot_binned_kernel<V, I><<<(unsigned)units, RB_THREADS, 0, s>>>(a, d, bv, L, partial);
            timer_after(s);
            return finish_dot<V>(s, partial, slots, result_host);
        }
        const int64_t nrb = ceil_div(a.outer_n, RB_THREADS);
        PlanRows L{};
        int64_t units = nrb;
        if (plan && plan->nat.nlong > 0) {  // natural order: the natural chunk set
            if (plan->outer_n != a.outer_n || plan->nnz != nnz)
                return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
            L = plan_rows(plan->nat);
            units += ceil_div(plan->nat.nchunks, RB_WARPS);
        }
        slots = units * RB_WARPS;
        if (units > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many outer entries");
        if (units > 0) {
            timer_before(s);
            dot_compressed_kernel<V, I><<<(unsigned)units, RB_THREADS, 0, s>>>(a, d, nrb, L, partial);
            timer_after(s);
        }
    }
    return finish_dot<V>(s, partial, slots, result_host);
}

#define GSA_INST_DOT(V, I)                                                                        \
    template size_t dot_workspace_size<V, I>(int, int64_t, const Plan *);                         \
    template int launch_dot<V, I>(cudaStream_t, int, int, int64_t, int64_t, int64_t, const I *,    \
                                  const I *, const V *, int, const V *, const V *, const Plan *,   \
                                  void *, size_t, void *);
GSA_INST_DOT(float, int32_t)
GSA_INST_DOT(float, int64_t)
GSA_INST_DOT(double, int32_t)
GSA_INST_DOT(double, int64_t)
GSA_INST_DOT(cf32, int32_t)
GSA_INST_DOT(cf32, int64_t)
GSA_INST_DOT(cf64, int32_t)
GSA_INST_DOT(cf64, int64_t)
GSA_INST_DOT(int32_t, int32_t)
GSA_INST_DOT(int32_t, int64_t)
GSA_INST_DOT(int64_t, int32_t)
GSA_INST_DOT(int64_t, int64_t)

}  // namespace gsa
