// Row-block gather: C[o, c] = beta*C[o, c] + alpha * sum_j a_j * op(B)(idx_j, c)
// -- kernel_spmatmul_csr_N! (src/matrix_csr/matrix_csr_kernels.jl:1-22) and
// kernel_spmatmul_csc_T! (src/matrix_csc/matrix_csc_kernels.jl:24-45).
//
// Each CTA of 256 threads owns 256 consecutive outer entries (rows), one per
// thread.  A row of at most SHORT_LEN entries is summed by its own thread with
// plain loads straight from HBM: neighbouring threads read neighbouring entries,
// so a warp's loads fall on the same cache lines and L1 merges them, and with
// tens of thousands of small CTAs in flight the GPU keeps enough loads
// outstanding to cover DRAM latency without staging.  A longer row is summed by
// the warp of the thread that owns it (lanes stride the row, a fixed shuffle
// tree reduces).  Entry loads are issued UNROLL at a time before their gathers,
// so each thread has several independent loads in flight.  No barriers, no
// workspace, no atomics; every row's summation order is fixed (deterministic).
//
// KC right-hand-side columns are accumulated per pass (SpMM); wider products
// loop over column chunks and re-read the row (L1/L2 hits).
#include "gsa_internal.cuh"

namespace gsa {

constexpr int RB_THREADS = 256;
constexpr int SHORT_LEN = 16;   // thread-per-row limit
constexpr int UNROLL = 4;       // entries loaded together per thread

// acc[c] += sum over j = jb, jb+S, ... < je of conj?(a_j) * op(B)(idx_j, c0 + c), in j order.
template <typename V, typename I, int KC, int S>
__device__ __forceinline__ void accumulate_range(const CompressedArgs<V, I> &a, const DenseIn<V> &B,
                                                 int64_t jb, int64_t je, int64_t c0, int64_t k,
                                                 V (&acc)[KC]) {
    const I *__restrict__ idx = a.idx;
    const V *__restrict__ val = a.val;
    const uint64_t inner = (uint64_t)a.inner_n;
    int64_t j = jb;
    for (; j + (UNROLL - 1) * S < je; j += UNROLL * S) {
        int64_t ci[UNROLL];
        V av[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            ci[u] = (int64_t)idx[j + u * S] - a.base;
            av[u] = conj_if(val[j + u * S], a.conjA);
        }
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
            const bool ok = (uint64_t)ci[u] < inner;
#pragma unroll
            for (int c = 0; c < KC; ++c)
                if (KC == 1 || c0 + c < k) {
                    const V xv = ok ? B.at(ci[u], c0 + c) : VT<V>::zero();
                    acc[c] = add(acc[c], mul(av[u], xv));
                }
        }
    }
    for (; j < je; j += S) {
        const int64_t c1 = (int64_t)idx[j] - a.base;
        const bool ok = (uint64_t)c1 < inner;
        const V av = conj_if(val[j], a.conjA);
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (KC == 1 || c0 + c < k) {
                const V xv = ok ? B.at(c1, c0 + c) : VT<V>::zero();
                acc[c] = add(acc[c], mul(av, xv));
            }
    }
}

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS)
rowblock_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C) {
    const int lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * RB_THREADS + threadIdx.x;
    int64_t b = 0, e = 0;
    if (r < a.outer_n) {
        b = (int64_t)__ldg(a.ptr + r) - a.base;
        e = (int64_t)__ldg(a.ptr + r + 1) - a.base;
        b = b < 0 ? 0 : (b > a.nnz ? a.nnz : b);
        e = e < b ? b : (e > a.nnz ? a.nnz : e);
    }
    const int64_t len = e - b;

    // ---- rows of at most SHORT_LEN entries: one thread each
    if (r < a.outer_n && len <= SHORT_LEN) {
        for (int64_t c0 = 0; c0 < k; c0 += KC) {
            V acc[KC];
#pragma unroll
            for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
            accumulate_range<V, I, KC, 1>(a, B, b, e, c0, k, acc);
#pragma unroll
            for (int c = 0; c < KC; ++c)
                if (KC == 1 || c0 + c < k) C.store(r, c0 + c, acc[c]);
        }
    }

    // ---- longer rows: the owning warp, one row at a time
    unsigned todo = __ballot_sync(0xffffffffu, r < a.outer_n && len > SHORT_LEN);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        const int64_t row = __shfl_sync(0xffffffffu, r, src);
        const int64_t rb = __shfl_sync(0xffffffffu, b, src);
        const int64_t re = __shfl_sync(0xffffffffu, e, src);
        for (int64_t c0 = 0; c0 < k; c0 += KC) {
            V acc[KC];
#pragma unroll
            for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
            accumulate_range<V, I, KC, 32>(a, B, rb + lane, re, c0, k, acc);
#pragma unroll
            for (int c = 0; c < KC; ++c) {
#pragma unroll
                for (int m = 16; m > 0; m >>= 1) acc[c] = add(acc[c], shfl_xor(acc[c], m));
            }
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < KC; ++c)
                    if (KC == 1 || c0 + c < k) C.store(row, c0 + c, acc[c]);
            }
        }
    }
}

template <typename V, typename I>
int launch_rowblock(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                    DenseOut<V> C) {
    if (a.outer_n == 0 || k == 0) return GSA_OK;
    const int64_t blocks = ceil_div(a.outer_n, RB_THREADS);
    if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many rows");
    constexpr int KW = sizeof(V) >= 16 ? 8 : 16;  // columns per pass for SpMM
    timer_before(s);
    if (k == 1) rowblock_kernel<V, I, 1><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C);
    else if (k <= 4) rowblock_kernel<V, I, 4><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C);
    else rowblock_kernel<V, I, KW><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "rowblock_kernel");
}

#define GSA_INST_RB(V, I)                                                                       \
    template int launch_rowblock<V, I>(cudaStream_t, const CompressedArgs<V, I> &, int64_t,     \
                                       DenseIn<V>, DenseOut<V>);
GSA_INST_RB(float, int32_t)
GSA_INST_RB(float, int64_t)
GSA_INST_RB(double, int32_t)
GSA_INST_RB(double, int64_t)
GSA_INST_RB(cf32, int32_t)
GSA_INST_RB(cf32, int64_t)
GSA_INST_RB(cf64, int32_t)
GSA_INST_RB(cf64, int64_t)
GSA_INST_RB(int32_t, int32_t)
GSA_INST_RB(int32_t, int64_t)
GSA_INST_RB(int64_t, int32_t)
GSA_INST_RB(int64_t, int64_t)

}  // namespace gsa
