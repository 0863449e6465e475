// Sparse x sparse products (SpGEMM).
//
// The reference (kernel_count_nnz_spgemm_csr! / kernel_spgemm_csr!,
// src/matrix_csr/matrix_csr_kernels.jl:250-343, and the CSC pair at
// src/matrix_csc/matrix_csc_kernels.jl:255-345) gives every output row a dense accumulator of
// the full output width: for each stored A[i,k] in storage order and each stored B[k,j] in
// storage order, acc[j] += A[i,k] * B[k,j]; then every reached position is stored, in column
// order, zero sums included.  That is m * n workspace.  Here each output row's products are
// expanded in the same order and summed per column in that order -- so every entry gets the
// reference's bits -- without a dense accumulator:
//   1. entry_flops_kernel: products of every stored entry of P (the length of the Q row it
//      selects); one scan; row_flops_kernel: products per output row from the scan at the row
//      pointers, rows listed as tiny, small or big.
//   2. tiny rows (at most 32 products), a thread each (tiny_kernel), and small rows (at most
//      256), a warp each (small_kernel): the row's products (column, value) expanded into
//      shared memory in order; a product is the first of its column when no earlier one has
//      the column; the count of first products is the row's entry count (symbolic pass); its
//      position is the number of first products of smaller columns and its value the in-order
//      sum of the products of its column, starting from zero (numeric pass).
//   3. big rows: expanded into global memory (expand_kernel: a CTA per row, 256 P entries at a
//      time, products spread evenly over the threads by a search of the chunk's offsets) with
//      keys row << cb | column, sorted by the library's stable LSD radix sort (the expansion is
//      in row order and in the reference's order within a row, so equal keys keep it), and
//      summed run by run in order.
// P and Q: CSR C = A * B runs over A's rows (P = A, Q = B); CSC C = A * B over B's columns
// (P = B, Q = A).  Products are A-value times B-value with Julia's arithmetic (separate
// multiply and add, textbook complex product), so the sums are the reference's bit for bit.
#include <type_traits>

#include "gsa_internal.cuh"

struct gsa_spgemm {
    int dtype = 0, itype = 0, csr = 1, base = 1;
    int64_t outer_n = 0, width = 0, q_outer = 0;
    const void *pp = nullptr, *pi = nullptr, *pv = nullptr;  // P: pointers, indices, values
    const void *qp = nullptr, *qi = nullptr, *qv = nullptr;  // Q
    int64_t nnz_c = 0;
    uint32_t ntiny = 0, nsmall = 0, nbig = 0;
    uint64_t pbig = 0;          // products of the big rows
    void *mem = nullptr;        // per-row arrays
    void *big = nullptr;        // big-row expansion and sort
    size_t cnt_off = 0, cptr_off = 0, tiny_off = 0, small_off = 0, big_off = 0, counters_off = 0;
    size_t boff_off = 0, keys_off = 0, flags_off = 0, rpos_off = 0, sums_off = 0;
    int cb = 0;                 // column bits of the big-row sort keys
};

namespace gsa {
namespace {

constexpr int SG_TINY_P = 32;     // products a thread sums in shared memory
constexpr int SG_TINY_WARPS = 2;
constexpr int SG_TINY_A = 8;      // A entries of a tiny row whose loads are issued together
constexpr int SG_WARP_P = 256;    // products a warp sums in shared memory
constexpr int SG_THREADS = 128;   // 4 warps
constexpr int SG_WARPS = SG_THREADS / 32;
constexpr int EX_THREADS_SG = 256;

// Julia's product: separate rounding of every multiply and add (the library is built without
// contraction), complex by the textbook formula.
__device__ __forceinline__ float jmul(float a, float b) { return a * b; }
__device__ __forceinline__ double jmul(double a, double b) { return a * b; }
__device__ __forceinline__ cf32 jmul(cf32 a, cf32 b) {
    return cf32{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cf64 jmul(cf64 a, cf64 b) {
    return cf64{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ int32_t jmul(int32_t a, int32_t b) { return mul(a, b); }
__device__ __forceinline__ int64_t jmul(int64_t a, int64_t b) { return mul(a, b); }

// A-value times B-value: in CSR P holds A, in CSC Q does.
template <typename V>
__device__ __forceinline__ V product(V p, V q, bool csr) { return csr ? jmul(p, q) : jmul(q, p); }

__device__ __forceinline__ uint32_t lane_lt() {
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return lt;
}

// L[t] = products of P's stored entry t (the length of the Q outer entry it selects; 0 for an
// index outside Q), t < nnz_p; L[nnz_p] = 0.
// totals[0] += all products.
template <typename I>
__global__ void entry_flops_kernel(int64_t nnz_p, const I *__restrict__ pi, const I *__restrict__ qp, int64_t q_outer,
                                   int base, uint32_t *__restrict__ L, unsigned long long *__restrict__ totals) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long sum = 0;  // one reduction and atomic per warp at the end
#pragma unroll 4
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= nnz_p; t += stride) {
        uint32_t len = 0;
        if (t < nnz_p) {
            const int64_t k = (int64_t)__ldg(pi + t) - base;
            if ((uint64_t)k < (uint64_t)q_outer) len = (uint32_t)((int64_t)__ldg(qp + k + 1) - __ldg(qp + k));
        }
        L[t] = len;
        sum += len;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&totals[0], sum);
}

// Products per outer entry of P from the scanned entry counts (the host has checked that all
// products together number fewer than 2^32, so the scan does not wrap); rows listed small or
// big; counters: [2] tiny rows (at most 32 products), [0] small rows (at most 256), [1] big
// rows; totals[1]: big-row products.
template <typename I>
__global__ void row_flops_kernel(int64_t outer_n, const I *__restrict__ pp, int base, const uint32_t *__restrict__ S,
                                 uint32_t *__restrict__ cnt, uint32_t *__restrict__ tiny_list,
                                 uint32_t *__restrict__ small_list, uint32_t *__restrict__ big_list,
                                 uint32_t *__restrict__ counters, unsigned long long *__restrict__ totals) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t o0 = (int64_t)blockIdx.x * blockDim.x; o0 < outer_n; o0 += stride) {
        const int64_t o = o0 + threadIdx.x;
        const bool valid = o < outer_n;
        uint32_t f = 0;
        if (valid) {
            const int64_t b = (int64_t)__ldg(pp + o) - base, e = (int64_t)__ldg(pp + o + 1) - base;
            f = e > b ? S[e] - S[b] : 0u;
            cnt[o] = 0;
        }
        const bool is_tiny = valid && f > 0 && f <= (uint32_t)SG_TINY_P;
        const bool is_small = valid && f > (uint32_t)SG_TINY_P && f <= (uint32_t)SG_WARP_P;
        const bool is_big = valid && f > (uint32_t)SG_WARP_P;
        const unsigned ms = __ballot_sync(0xffffffffu, is_small), mb = __ballot_sync(0xffffffffu, is_big);
        const unsigned mt = __ballot_sync(0xffffffffu, is_tiny);
        const int lane = threadIdx.x & 31;
        const unsigned lt = lane_lt();
        unsigned long long fb = is_big ? f : 0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) fb += __shfl_xor_sync(0xffffffffu, fb, d);
        uint32_t bs = 0, bb = 0, bt = 0;
        if (lane == 0) {
            if (mt) bt = atomicAdd(&counters[2], (uint32_t)__popc(mt));
            if (ms) bs = atomicAdd(&counters[0], (uint32_t)__popc(ms));
            if (mb) bb = atomicAdd(&counters[1], (uint32_t)__popc(mb));
            if (fb) atomicAdd(&totals[1], fb);
        }
        bs = __shfl_sync(0xffffffffu, bs, 0);
        bb = __shfl_sync(0xffffffffu, bb, 0);
        bt = __shfl_sync(0xffffffffu, bt, 0);
        if (is_tiny) tiny_list[bt + __popc(mt & lt)] = (uint32_t)o;
        if (is_small) small_list[bs + __popc(ms & lt)] = (uint32_t)o;
        if (is_big) big_list[bb + __popc(mb & lt)] = (uint32_t)o;
    }
}


// Thread per listed tiny row (at most SG_TINY_P products): the same expansion, sums and
// positions as small_kernel, each thread in its own column of the warp's shared block
// (slot s of lane l at s * 32 + l, so the lanes never share a bank), the first products of
// each column kept as a bit mask.
template <typename V, typename I, bool NUMERIC>
__global__ void __launch_bounds__(SG_TINY_WARPS * 32)
tiny_kernel(const uint32_t *__restrict__ list, const uint32_t *__restrict__ counters, const I *__restrict__ pp,
            const I *__restrict__ pi, const V *__restrict__ pv, const I *__restrict__ qp, const I *__restrict__ qi,
            const V *__restrict__ qv, int64_t q_outer, int base, bool csr, uint32_t *__restrict__ cnt,
            const uint32_t *__restrict__ cptr, I *__restrict__ idx_out, V *__restrict__ val_out) {
    __shared__ uint32_t tj[SG_TINY_WARPS][SG_TINY_P * 32];
    __shared__ V tv[NUMERIC ? SG_TINY_WARPS : 1][NUMERIC ? SG_TINY_P * 32 : 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t nlisted = counters[2];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nlisted; q += gridDim.x * blockDim.x) {
        const uint32_t o = list[q];
        const int64_t b = (int64_t)__ldg(pp + o) - base, e = (int64_t)__ldg(pp + o + 1) - base;
        uint32_t P = 0;
        auto expand = [&](int64_t qb, uint32_t len, V a) {
#pragma unroll 4
            for (uint32_t u = 0; u < len; ++u) {
                if (P + u < (uint32_t)SG_TINY_P) {
                    tj[w][(P + u) * 32 + lane] = (uint32_t)((int64_t)__ldg(qi + qb + u) - base);
                    if constexpr (NUMERIC) tv[w][(P + u) * 32 + lane] = product(a, ldg(qv + qb + u), csr);
                }
            }
            P = P + len < (uint32_t)SG_TINY_P ? P + len : (uint32_t)SG_TINY_P;
        };
        if (e - b <= SG_TINY_A) {
            // rows of up to SG_TINY_A entries: their indices, Q-row bounds and values loaded
            // together first, so the loads overlap instead of forming one chain per entry
            int64_t qb[SG_TINY_A];
            uint32_t len[SG_TINY_A];
            V a[SG_TINY_A];
#pragma unroll
            for (int c = 0; c < SG_TINY_A; ++c) {
                const int64_t t = b + c;
                qb[c] = (int64_t)(t < e ? __ldg(pi + t) : (I)0) - base;  // k for now
                if constexpr (NUMERIC) a[c] = t < e ? ldg(pv + t) : V{};
            }
#pragma unroll
            for (int c = 0; c < SG_TINY_A; ++c) {
                const int64_t k = qb[c];
                const bool ok = b + c < e && (uint64_t)k < (uint64_t)q_outer;
                const int64_t q0 = ok ? (int64_t)__ldg(qp + k) - base : 0;
                len[c] = ok ? (uint32_t)((int64_t)__ldg(qp + k + 1) - base - q0) : 0u;
                qb[c] = q0;
            }
#pragma unroll
            for (int c = 0; c < SG_TINY_A; ++c)
                if (len[c]) expand(qb[c], len[c], NUMERIC ? a[c] : V{});
            // The products are SG_TINY_A runs, one per A entry, in A order.  When every run is
            // sorted by column (sorted Q rows), a merge of the runs visits the columns in
            // increasing order and, for each, its products in the reference's order (runs in A
            // order, each run in its own order): no quadratic scan.
            uint32_t hs[SG_TINY_A], he[SG_TINY_A];
            uint32_t off = 0;
            bool sorted = true;
#pragma unroll
            for (int c = 0; c < SG_TINY_A; ++c) {
                hs[c] = off < P ? off : P;
                off += len[c];
                he[c] = off < P ? off : P;
                for (uint32_t u = hs[c] + 1; u < he[c]; ++u)
                    if (tj[w][u * 32 + lane] < tj[w][(u - 1) * 32 + lane]) sorted = false;
            }
            if (sorted) {
                uint64_t jc[SG_TINY_A];
#pragma unroll
                for (int c = 0; c < SG_TINY_A; ++c) jc[c] = hs[c] < he[c] ? tj[w][hs[c] * 32 + lane] : ~0ull;
                const uint32_t out0 = NUMERIC ? cptr[o] : 0;
                uint32_t count = 0;
                for (uint32_t guard = 0; guard <= (uint32_t)SG_TINY_P; ++guard) {
                    uint64_t jmin = jc[0];
#pragma unroll
                    for (int c = 1; c < SG_TINY_A; ++c) jmin = jc[c] < jmin ? jc[c] : jmin;
                    if (jmin == ~0ull) break;
                    V acc = VT<V>::zero();
#pragma unroll
                    for (int c = 0; c < SG_TINY_A; ++c) {
                        while (jc[c] == jmin) {
                            if constexpr (NUMERIC) acc = add(acc, tv[w][hs[c] * 32 + lane]);
                            ++hs[c];
                            jc[c] = hs[c] < he[c] ? tj[w][hs[c] * 32 + lane] : ~0ull;
                        }
                    }
                    if constexpr (NUMERIC) {
                        idx_out[out0 + count] = (I)((int64_t)jmin + base);
                        val_out[out0 + count] = acc;
                    }
                    ++count;
                }
                if constexpr (!NUMERIC) cnt[o] = count;
                continue;
            }
        } else {
            for (int64_t t = b; t < e; ++t) {
                const int64_t k = (int64_t)__ldg(pi + t) - base;
                if ((uint64_t)k >= (uint64_t)q_outer) continue;
                const int64_t q0 = (int64_t)__ldg(qp + k) - base;
                const uint32_t l = (uint32_t)((int64_t)__ldg(qp + k + 1) - base - q0);
                V av{};
                if constexpr (NUMERIC) av = ldg(pv + t);
                expand(q0, l, av);
            }
        }
        uint32_t firsts = 0;
        for (uint32_t s2 = 0; s2 < P; ++s2) {
            const uint32_t j = tj[w][s2 * 32 + lane];
            bool first = true;
            for (uint32_t t = 0; t < s2; ++t)
                if (tj[w][t * 32 + lane] == j) {
                    first = false;
                    break;
                }
            if (first) firsts |= 1u << s2;
        }
        if constexpr (!NUMERIC) {
            cnt[o] = (uint32_t)__popc(firsts);
        } else {
            const uint32_t out0 = cptr[o];
            for (uint32_t rest = firsts; rest; rest &= rest - 1) {
                const uint32_t s2 = (uint32_t)(__ffs(rest) - 1);
                const uint32_t j = tj[w][s2 * 32 + lane];
                uint32_t pos = 0;
                V acc = VT<V>::zero();
                for (uint32_t t = 0; t < P; ++t) {
                    const uint32_t jt = tj[w][t * 32 + lane];
                    pos += (((firsts >> t) & 1u) && jt < j) ? 1u : 0u;
                    if (t >= s2 && jt == j) acc = add(acc, tv[w][t * 32 + lane]);
                }
                idx_out[out0 + pos] = (I)((int64_t)j + base);
                val_out[out0 + pos] = acc;
            }
        }
    }
}

// Warp per listed small row (at most SG_WARP_P products).  The row's products go to shared
// memory in the reference's order (P entries in storage order, each Q row in storage order):
// the lanes take 32 P entries at a time, scan their Q-row lengths for the offsets, and write
// their own rows as keys column << 8 | slot (values by slot).  A warp bitonic sort of the keys
// puts each column's products together in slot order; run starts are the entries (symbolic:
// cnt[o] = runs), their scanned count the positions, and each run is summed in order from zero
// (numeric, written from cptr[o]).
template <typename V, typename I, bool NUMERIC>
__global__ void __launch_bounds__(SG_THREADS)
small_kernel(const uint32_t *__restrict__ list, const uint32_t *__restrict__ counters, const I *__restrict__ pp,
             const I *__restrict__ pi, const V *__restrict__ pv, const I *__restrict__ qp, const I *__restrict__ qi,
             const V *__restrict__ qv, int64_t q_outer, int base, bool csr, uint32_t *__restrict__ cnt,
             const uint32_t *__restrict__ cptr, I *__restrict__ idx_out, V *__restrict__ val_out) {
    __shared__ uint64_t sk[SG_WARPS][SG_WARP_P];
    __shared__ V sv[NUMERIC ? SG_WARPS : 1][NUMERIC ? SG_WARP_P : 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = lane_lt();
    const uint32_t nlisted = counters[0];
    for (uint32_t q = blockIdx.x * SG_WARPS + w; q < nlisted; q += gridDim.x * SG_WARPS) {
        const uint32_t o = list[q];
        const int64_t b = (int64_t)__ldg(pp + o) - base, e = (int64_t)__ldg(pp + o + 1) - base;
        uint32_t P = 0;
        for (int64_t c0 = b; c0 < e; c0 += 32) {
            const int64_t t = c0 + lane;
            uint32_t len = 0;
            int64_t qb = 0;
            V a{};
            if (t < e) {
                const int64_t k = (int64_t)__ldg(pi + t) - base;
                if ((uint64_t)k < (uint64_t)q_outer) {
                    qb = (int64_t)__ldg(qp + k) - base;
                    len = (uint32_t)((int64_t)__ldg(qp + k + 1) - base - qb);
                    if (NUMERIC) a = ldg(pv + t);
                }
            }
            uint32_t off = len;  // inclusive scan, then exclusive
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, off, d);
                if (lane >= d) off += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, off, 31);
            off -= len;
            // the row has at most SG_WARP_P products (its flops), so every slot is in range;
            // the bound also holds for a malformed structure
            for (uint32_t u = 0; u < len && P + off + u < (uint32_t)SG_WARP_P; ++u) {
                const uint32_t slot = P + off + u;
                const uint64_t j = (uint32_t)((int64_t)__ldg(qi + qb + u) - base);
                sk[w][slot] = (j << 8) | slot;
                if constexpr (NUMERIC) sv[w][slot] = product(a, ldg(qv + qb + u), csr);
            }
            P += total;
        }
        if (P > (uint32_t)SG_WARP_P) P = SG_WARP_P;
        uint32_t P2 = 32;
        while (P2 < P) P2 <<= 1;
        for (uint32_t i = P + lane; i < P2; i += 32) sk[w][i] = ~0ull;
        __syncwarp();
        for (uint32_t kk = 2; kk <= P2; kk <<= 1) {
            for (uint32_t jj = kk >> 1; jj > 0; jj >>= 1) {
                for (uint32_t i = lane; i < P2; i += 32) {
                    const uint32_t ixj = i ^ jj;
                    if (ixj > i) {
                        const uint64_t x = sk[w][i], y = sk[w][ixj];
                        if ((x > y) == ((i & kk) == 0)) {
                            sk[w][i] = y;
                            sk[w][ixj] = x;
                        }
                    }
                }
                __syncwarp();
            }
        }
        uint32_t before = 0;  // run starts in earlier passes of the loop below
        const uint32_t out0 = NUMERIC ? cptr[o] : 0;
        for (uint32_t i0 = 0; i0 < P; i0 += 32) {
            const uint32_t i = i0 + lane;
            bool start = false;
            if (i < P) start = i == 0 || (sk[w][i] >> 8) != (sk[w][i - 1] >> 8);
            const unsigned ms = __ballot_sync(0xffffffffu, start);
            if constexpr (NUMERIC) {
                if (start) {
                    const uint64_t j = sk[w][i] >> 8;
                    V acc = VT<V>::zero();
                    for (uint32_t u = i; u < P && (sk[w][u] >> 8) == j; ++u) acc = add(acc, sv[w][sk[w][u] & 0xffu]);
                    const uint32_t pos = before + __popc(ms & lt);
                    idx_out[out0 + pos] = (I)((int64_t)j + base);
                    val_out[out0 + pos] = acc;
                }
            }
            before += __popc(ms);
        }
        if constexpr (!NUMERIC) {
            if (lane == 0) cnt[o] = before;
        }
        __syncwarp();
    }
}

// ---- big rows ----------------------------------------------------------------

// flops of each big row, for the scan of their expansion offsets
template <typename I>
__global__ void big_flops_kernel(const uint32_t *__restrict__ list, uint32_t nbig, const I *__restrict__ pp, int base,
                                 const uint32_t *__restrict__ S, uint32_t *__restrict__ bflops) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q <= nbig; q += gridDim.x * blockDim.x) {
        uint32_t f = 0;
        if (q < nbig) {
            const uint32_t o = list[q];
            f = S[(int64_t)__ldg(pp + o + 1) - base] - S[(int64_t)__ldg(pp + o) - base];
        }
        bflops[q] = f;
    }
}

// CTA per big row: its products written from boff[q], in the reference's order, as key
// (q << cb | column), position and value.  256 P entries at a time: their Q-row lengths are scanned, then
// product p of the chunk goes to thread p mod 256, which finds its P entry by a binary search
// of the chunk's offsets.
template <typename V, typename I>
__global__ void __launch_bounds__(EX_THREADS_SG)
expand_kernel(const uint32_t *__restrict__ list, uint32_t nbig, const uint32_t *__restrict__ boff,
              const I *__restrict__ pp, const I *__restrict__ pi, const V *__restrict__ pv, const I *__restrict__ qp,
              const I *__restrict__ qi, const V *__restrict__ qv, int64_t q_outer, int base, bool csr, int cb,
              uint64_t *__restrict__ ex_key, uint32_t *__restrict__ ex_pos, V *__restrict__ ex_val) {
    constexpr int T = EX_THREADS_SG;
    __shared__ uint32_t s_off[T + 1];
    __shared__ int64_t s_qb[T];
    __shared__ V s_a[T];
    __shared__ uint32_t s_wsum[T / 32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
        const uint32_t o = list[q];
        const int64_t b = (int64_t)__ldg(pp + o) - base, e = (int64_t)__ldg(pp + o + 1) - base;
        uint32_t run = boff[q];
        for (int64_t c0 = b; c0 < e; c0 += T) {
            const int64_t t = c0 + tid;
            uint32_t len = 0;
            int64_t qb = 0;
            V a{};
            if (t < e) {
                const int64_t k = (int64_t)__ldg(pi + t) - base;
                if ((uint64_t)k < (uint64_t)q_outer) {
                    qb = (int64_t)__ldg(qp + k) - base;
                    len = (uint32_t)((int64_t)__ldg(qp + k + 1) - base - qb);
                    a = ldg(pv + t);
                }
            }
            s_qb[tid] = qb;
            s_a[tid] = a;
            uint32_t x = len;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += y;
            }
            if (lane == 31) s_wsum[w] = x;
            __syncthreads();
            uint32_t before = 0;
            for (int v = 0; v < w; ++v) before += s_wsum[v];
            s_off[tid] = before + x - len;
            if (tid == T - 1) s_off[T] = before + x;
            __syncthreads();
            const uint32_t total = s_off[T];
            for (uint32_t p = tid; p < total; p += T) {
                int lo = 0, hi = T - 1;  // the last entry whose offset is <= p
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_off[mid] <= p) lo = mid;
                    else hi = mid - 1;
                }
                const int64_t f = s_qb[lo] + (p - s_off[lo]);
                const uint32_t slot = run + p;
                // masked to its field, so that an index outside the matrix cannot reach the row bits
                const uint64_t col = (uint64_t)((int64_t)__ldg(qi + f) - base) & ((1ull << cb) - 1);
                ex_key[slot] = ((uint64_t)q << cb) | col;
                ex_pos[slot] = slot;
                ex_val[slot] = product(s_a[lo], ldg(qv + f), csr);
            }
            run += total;
            __syncthreads();
        }
    }
}

// One thread per run of equal keys: the in-order sum from zero; flags[i] = 1 at run starts.
template <typename V>
__global__ void big_runs_kernel(int64_t total, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ perm,
                                const V *__restrict__ ex_val, V *__restrict__ sums, uint32_t *__restrict__ flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= total; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        if (i < total) {
            const uint64_t k = keys[i];
            if (i == 0 || keys[i - 1] != k) {
                V acc = VT<V>::zero();
                for (int64_t t = i; t < total && keys[t] == k; ++t) acc = add(acc, ldg(ex_val + perm[t]));
                sums[i] = acc;
                f = 1;
            }
        }
        flags[i] = f;
    }
}

// Entries of each big row: the run starts in its range of the sorted products (sorting by
// (row, column) keeps every row in the range its expansion had).
__global__ void big_count_kernel(const uint32_t *__restrict__ list, uint32_t nbig, const uint32_t *__restrict__ boff,
                                 const uint32_t *__restrict__ rpos, uint32_t *__restrict__ cnt) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nbig; q += gridDim.x * blockDim.x)
        cnt[list[q]] = rpos[boff[q + 1]] - rpos[boff[q]];
}

template <typename V, typename I>
__global__ void big_write_kernel(int64_t total, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ flags,
                                 const uint32_t *__restrict__ rpos, const V *__restrict__ sums,
                                 const uint32_t *__restrict__ list, const uint32_t *__restrict__ boff, int cb,
                                 const uint32_t *__restrict__ cptr, int base, I *__restrict__ idx_out,
                                 V *__restrict__ val_out) {
    const uint64_t mask = cb >= 64 ? ~0ull : ((1ull << cb) - 1);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flags[i]) continue;
        const uint64_t k = keys[i];
        const uint32_t q = (uint32_t)(k >> cb);
        const uint32_t out = cptr[list[q]] + (rpos[i] - rpos[boff[q]]);
        idx_out[out] = (I)((int64_t)(k & mask) + base);
        val_out[out] = sums[i];
    }
}

template <typename I>
__global__ void pointers_kernel(int64_t outer_n, const uint32_t *__restrict__ cptr, int base, I *__restrict__ ptr_out) {
    for (int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; o <= outer_n; o += (int64_t)gridDim.x * blockDim.x)
        ptr_out[o] = (I)((int64_t)cptr[o] + base);
}

unsigned sg_grid(int64_t n, int64_t per_cta, int64_t cap) {
    int64_t b = ceil_div(n, per_cta);
    if (b > cap) b = cap;
    return (unsigned)(b > 0 ? b : 1);
}

// Per-row arrays of a product (one allocation): entry flops and their scan, row counts and
// their scan, the two row lists, counters and totals, scan scratch.
struct RowLayout {
    size_t L, cnt, cptr, tiny, small, big, counters, totals, bsums, bytes;
};
RowLayout row_layout(int64_t outer_n, int64_t nnz_p) {
    RowLayout R;
    Carver cv(nullptr);
    R.L = cv.reserve<uint32_t>(nnz_p + 1);
    R.cnt = cv.reserve<uint32_t>(outer_n + 2);
    R.cptr = cv.reserve<uint32_t>(outer_n + 2);
    R.tiny = cv.reserve<uint32_t>(outer_n > 0 ? outer_n : 1);
    R.small = cv.reserve<uint32_t>(outer_n > 0 ? outer_n : 1);
    R.big = cv.reserve<uint32_t>(outer_n > 0 ? outer_n : 1);
    R.counters = cv.reserve<uint32_t>(4);
    R.totals = cv.reserve<unsigned long long>(2);
    const int64_t ns = nnz_p + 1 > outer_n + 2 ? nnz_p + 1 : outer_n + 2;
    R.bsums = cv.reserve<uint32_t>(scan_block_sums(ns));
    R.bytes = align_up(cv.off, 256);
    return R;
}

// Big-row arrays, once their products are known.
struct BigLayout {
    size_t bflops, boff, exval, sort, flags, rpos, sums, bsums, bytes;
};
BigLayout big_layout(uint32_t nbig, uint64_t pbig, size_t vsize) {
    BigLayout B;
    Carver cv(nullptr);
    B.bflops = cv.reserve<uint32_t>((size_t)nbig + 1);
    B.boff = cv.reserve<uint32_t>((size_t)nbig + 1);
    B.exval = cv.reserve<unsigned char>(pbig * vsize);
    B.sort = cv.reserve<unsigned char>(radix_sort_workspace((int64_t)pbig));
    B.flags = cv.reserve<uint32_t>(pbig + 1);
    B.rpos = cv.reserve<uint32_t>(pbig + 1);
    B.sums = cv.reserve<unsigned char>(pbig * vsize);
    const uint64_t ns = pbig + 1 > (uint64_t)nbig + 1 ? pbig + 1 : (uint64_t)nbig + 1;
    B.bsums = cv.reserve<uint32_t>(scan_block_sums((int64_t)ns));
    B.bytes = align_up(cv.off, 256);
    return B;
}

int read_back(cudaStream_t s, void *host, const void *dev, size_t bytes, const char *what) {
    int rc = check_cuda(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s), what);
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), what);
    return rc;
}

}  // namespace

// Symbolic phase: counts, row pointers (written to ptr_c), big-row sums.
template <typename V, typename I>
int spgemm_create(cudaStream_t s, gsa_spgemm *h, int64_t nnz_p, I *ptr_c) {
    const I *pp = (const I *)h->pp, *pi = (const I *)h->pi, *qp = (const I *)h->qp, *qi = (const I *)h->qi;
    const V *pv = (const V *)h->pv, *qv = (const V *)h->qv;
    const int64_t outer_n = h->outer_n;
    const RowLayout R = row_layout(outer_n, nnz_p);
    int rc = check_cuda(cudaMalloc(&h->mem, R.bytes), "spgemm: row arrays");
    if (rc) return rc;
    char *m = (char *)h->mem;
    uint32_t *L = (uint32_t *)(m + R.L), *cnt = (uint32_t *)(m + R.cnt), *cptr = (uint32_t *)(m + R.cptr);
    uint32_t *tiny = (uint32_t *)(m + R.tiny), *small = (uint32_t *)(m + R.small), *big = (uint32_t *)(m + R.big);
    uint32_t *counters = (uint32_t *)(m + R.counters), *bsums = (uint32_t *)(m + R.bsums);
    unsigned long long *totals = (unsigned long long *)(m + R.totals);
    h->cnt_off = R.cnt;
    h->cptr_off = R.cptr;
    h->tiny_off = R.tiny;
    h->small_off = R.small;
    h->big_off = R.big;
    h->counters_off = R.counters;
    rc = check_cuda(cudaMemsetAsync(counters, 0, 4 * sizeof(uint32_t), s), "spgemm: clear");
    if (!rc) rc = check_cuda(cudaMemsetAsync(totals, 0, 2 * sizeof(unsigned long long), s), "spgemm: clear");
    if (!rc) rc = check_cuda(cudaMemsetAsync(cnt, 0, (size_t)(outer_n + 2) * sizeof(uint32_t), s), "spgemm: clear");
    if (rc) return rc;
    entry_flops_kernel<I><<<sg_grid(nnz_p + 1, 256, 152 * 32), 256, 0, s>>>(nnz_p, pi, qp, h->q_outer, h->base, L,
                                                                            totals);
    rc = check_cuda(cudaGetLastError(), "spgemm: entry_flops_kernel");
    unsigned long long tot[2] = {0, 0};
    if (!rc) rc = read_back(s, tot, totals, sizeof(tot), "spgemm: product count");
    if (rc) return rc;
    if (tot[0] >= 0xffffffffull)
        return fail(GSA_ERR_UNSUPPORTED, "the product has %llu products; at most 2^32 - 2 are supported", tot[0]);
    rc = scan_u32(s, L, L, nnz_p + 1, bsums);
    if (rc) return rc;
    if (outer_n > 0)
        row_flops_kernel<I><<<sg_grid(outer_n, 256, 152 * 32), 256, 0, s>>>(outer_n, pp, h->base, L, cnt, tiny, small, big,
                                                                          counters, totals);
    rc = check_cuda(cudaGetLastError(), "spgemm: row_flops_kernel");
    uint32_t ctr[4] = {0, 0, 0, 0};
    if (!rc) rc = read_back(s, ctr, counters, sizeof(ctr), "spgemm: row lists");
    if (!rc) rc = read_back(s, tot, totals, sizeof(tot), "spgemm: big-row products");
    if (rc) return rc;
    h->nsmall = ctr[0];
    h->nbig = ctr[1];
    h->ntiny = ctr[2];
    if (h->ntiny)
        tiny_kernel<V, I, false><<<sg_grid(h->ntiny, SG_TINY_WARPS * 32, 152 * 32), SG_TINY_WARPS * 32, 0, s>>>(
            tiny, counters, pp, pi, pv, qp, qi, qv, h->q_outer, h->base, h->csr != 0, cnt, nullptr, nullptr, nullptr);
    rc = check_cuda(cudaGetLastError(), "spgemm: tiny_kernel");
    if (rc) return rc;
    h->pbig = tot[1];
    if (h->nsmall)
        small_kernel<V, I, false><<<sg_grid(h->nsmall, SG_WARPS, 152 * 16), SG_THREADS, 0, s>>>(
            small, counters, pp, pi, pv, qp, qi, qv, h->q_outer, h->base, h->csr != 0, cnt, nullptr, nullptr, nullptr);
    rc = check_cuda(cudaGetLastError(), "spgemm: small_kernel");
    if (rc) return rc;
    if (h->nbig) {
        const BigLayout B = big_layout(h->nbig, h->pbig, sizeof(V));
        rc = check_cuda(cudaMalloc(&h->big, B.bytes), "spgemm: big-row arrays");
        if (rc) return rc;
        char *g = (char *)h->big;
        h->flags_off = B.flags;
        h->rpos_off = B.rpos;
        h->sums_off = B.sums;
        h->boff_off = B.boff;
        h->cb = radix_bits_for(h->width);
        const int qb = radix_bits_for(h->nbig);
        uint32_t *bflops = (uint32_t *)(g + B.bflops), *boff = (uint32_t *)(g + B.boff);
        V *exval = (V *)(g + B.exval), *sums = (V *)(g + B.sums);
        uint32_t *flags = (uint32_t *)(g + B.flags);
        uint32_t *rpos = (uint32_t *)(g + B.rpos), *gbsums = (uint32_t *)(g + B.bsums);
        uint64_t *exkey;
        uint32_t *expos;
        radix_sort_inputs(g + B.sort, (int64_t)h->pbig, &exkey, &expos);
        big_flops_kernel<I><<<sg_grid((int64_t)h->nbig + 1, 256, 152 * 8), 256, 0, s>>>(big, h->nbig, pp, h->base, L,
                                                                                       bflops);
        rc = check_cuda(cudaGetLastError(), "spgemm: big_flops_kernel");
        if (!rc) rc = scan_u32(s, bflops, boff, (int64_t)h->nbig + 1, gbsums);
        if (rc) return rc;
        expand_kernel<V, I><<<sg_grid(h->nbig, 1, 152 * 4), EX_THREADS_SG, 0, s>>>(
            big, h->nbig, boff, pp, pi, pv, qp, qi, qv, h->q_outer, h->base, h->csr != 0, h->cb, exkey, expos, exval);
        rc = check_cuda(cudaGetLastError(), "spgemm: expand_kernel");
        if (rc) return rc;
        // stable by (row, column): the expansion is in row order and, within a row, in the
        // reference's order, so equal columns keep that order
        uint64_t *keys;
        uint32_t *perm;
        rc = radix_sort_pairs(s, g + B.sort, (int64_t)h->pbig, h->cb + qb, &keys, &perm);
        if (rc) return rc;
        h->keys_off = (size_t)((char *)keys - g);
        big_runs_kernel<V><<<sg_grid((int64_t)h->pbig + 1, 256, 152 * 32), 256, 0, s>>>((int64_t)h->pbig, keys, perm,
                                                                                        exval, sums, flags);
        rc = check_cuda(cudaGetLastError(), "spgemm: big_runs_kernel");
        if (!rc) rc = scan_u32(s, flags, rpos, (int64_t)h->pbig + 1, gbsums);
        if (rc) return rc;
        big_count_kernel<<<sg_grid(h->nbig, 256, 152 * 8), 256, 0, s>>>(big, h->nbig, boff, rpos, cnt);
        rc = check_cuda(cudaGetLastError(), "spgemm: big_count_kernel");
        if (rc) return rc;
    }
    rc = scan_u32(s, cnt, cptr, outer_n + 1, bsums);
    if (rc) return rc;
    uint32_t total = 0;
    rc = read_back(s, &total, cptr + outer_n, sizeof(total), "spgemm: entry count");
    if (rc) return rc;
    if (sizeof(I) == 4 && (int64_t)total + h->base > 0x7fffffffLL)  // checked before any pointer is written
        return fail(GSA_ERR_UNSUPPORTED, "the product has %u entries, more than Int32 pointers can address", total);
    pointers_kernel<I><<<sg_grid(outer_n + 1, 256, 152 * 8), 256, 0, s>>>(outer_n, cptr, h->base, ptr_c);
    rc = check_cuda(cudaGetLastError(), "spgemm: pointers_kernel");
    if (!rc) h->nnz_c = total;
    return rc;
}

// Numeric phase: the entries of the small rows, then those of the big rows.
template <typename V, typename I>
int spgemm_compute(cudaStream_t s, const gsa_spgemm *h, I *idx_c, V *val_c) {
    const char *m = (const char *)h->mem;
    const uint32_t *cptr = (const uint32_t *)(m + h->cptr_off);
    const uint32_t *small = (const uint32_t *)(m + h->small_off), *big = (const uint32_t *)(m + h->big_off);
    const uint32_t *tiny = (const uint32_t *)(m + h->tiny_off);
    const uint32_t *counters = (const uint32_t *)(m + h->counters_off);
    if (h->ntiny)
        tiny_kernel<V, I, true><<<sg_grid(h->ntiny, SG_TINY_WARPS * 32, 152 * 32), SG_TINY_WARPS * 32, 0, s>>>(
            tiny, counters, (const I *)h->pp, (const I *)h->pi, (const V *)h->pv, (const I *)h->qp, (const I *)h->qi,
            (const V *)h->qv, h->q_outer, h->base, h->csr != 0, nullptr, cptr, idx_c, val_c);
    int rc = check_cuda(cudaGetLastError(), "spgemm: tiny_kernel");
    if (rc) return rc;
    if (h->nsmall)
        small_kernel<V, I, true><<<sg_grid(h->nsmall, SG_WARPS, 152 * 16), SG_THREADS, 0, s>>>(
            small, counters, (const I *)h->pp, (const I *)h->pi, (const V *)h->pv, (const I *)h->qp, (const I *)h->qi,
            (const V *)h->qv, h->q_outer, h->base, h->csr != 0, nullptr, cptr, idx_c, val_c);
    rc = check_cuda(cudaGetLastError(), "spgemm: small_kernel");
    if (rc || !h->nbig) return rc;
    const char *g = (const char *)h->big;
    big_write_kernel<V, I><<<sg_grid((int64_t)h->pbig, 256, 152 * 32), 256, 0, s>>>(
        (int64_t)h->pbig, (const uint64_t *)(g + h->keys_off), (const uint32_t *)(g + h->flags_off),
        (const uint32_t *)(g + h->rpos_off), (const V *)(g + h->sums_off), big,
        (const uint32_t *)(g + h->boff_off), h->cb, cptr, h->base, idx_c, val_c);
    return check_cuda(cudaGetLastError(), "spgemm: big_write_kernel");
}

}  // namespace gsa

namespace {
bool sg_misaligned(const void *p, size_t a) { return a && ((uintptr_t)p % a) != 0; }

struct SpgemmCreateBody {
    cudaStream_t s;
    gsa_spgemm *h;
    int64_t nnz_p;
    void *ptr_c;
    template <typename V, typename I> int operator()() {
        return gsa::spgemm_create<V, I>(s, h, nnz_p, (I *)ptr_c);
    }
};
struct SpgemmComputeBody {
    cudaStream_t s;
    const gsa_spgemm *h;
    void *idx_c, *val_c;
    template <typename V, typename I> int operator()() {
        return gsa::spgemm_compute<V, I>(s, h, (I *)idx_c, (V *)val_c);
    }
};
}  // namespace

extern "C" {

int gsa_spgemm_destroy(gsa_spgemm *handle) {
    if (!handle) return GSA_OK;
    int rc = GSA_OK;
    if (handle->big) rc = gsa::check_cuda(cudaFree(handle->big), "spgemm: free");
    if (handle->mem) {
        const int rc2 = gsa::check_cuda(cudaFree(handle->mem), "spgemm: free");
        if (!rc) rc = rc2;
    }
    delete handle;
    return rc;
}

int gsa_spgemm_create(void *stream, int format, int dtype, int itype, int64_t m, int64_t k, int64_t n,
                      const void *ptr_a, const void *idx_a, const void *val_a, int64_t nnz_a, const void *ptr_b,
                      const void *idx_b, const void *val_b, int64_t nnz_b, int base, void *ptr_c, int64_t *nnz_c,
                      gsa_spgemm **handle) {
    using namespace gsa;
    const size_t vs = dtype_size(dtype), is = itype_size(itype);
    if (!vs || !is) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (format != 0 && format != 1) return fail(GSA_ERR_INVALID_ARG, "format must be 0 (CSR) or 1 (CSC)");
    if (!handle || !nnz_c) return fail(GSA_ERR_INVALID_ARG, "handle / nnz_c is NULL");
    *handle = nullptr;
    if (m < 0 || k < 0 || n < 0 || nnz_a < 0 || nnz_b < 0) return fail(GSA_ERR_INVALID_ARG, "negative size");
    const bool csr = format == 0;
    const int64_t outer_n = csr ? m : n, width = csr ? n : m, nnz_p = csr ? nnz_a : nnz_b;
    if (outer_n >= 0xfffffffeLL || width > 0x100000000LL || k >= 0xfffffffeLL)
        return fail(GSA_ERR_UNSUPPORTED, "dimensions beyond 2^32 - 2 are not supported");
    if (!ptr_a || !ptr_b || !ptr_c) return fail(GSA_ERR_INVALID_ARG, "pointer arrays are NULL");
    if ((nnz_a > 0 && (!idx_a || !val_a)) || (nnz_b > 0 && (!idx_b || !val_b)))
        return fail(GSA_ERR_INVALID_ARG, "index / value arrays are NULL");
    if (sg_misaligned(ptr_a, is) || sg_misaligned(idx_a, is) || sg_misaligned(val_a, vs) || sg_misaligned(ptr_b, is) ||
        sg_misaligned(idx_b, is) || sg_misaligned(val_b, vs) || sg_misaligned(ptr_c, is))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    gsa_spgemm *h = new gsa_spgemm();
    h->dtype = dtype;
    h->itype = itype;
    h->csr = csr ? 1 : 0;
    h->base = base;
    h->outer_n = outer_n;
    h->width = width;
    h->q_outer = k;
    h->pp = csr ? ptr_a : ptr_b;
    h->pi = csr ? idx_a : idx_b;
    h->pv = csr ? val_a : val_b;
    h->qp = csr ? ptr_b : ptr_a;
    h->qi = csr ? idx_b : idx_a;
    h->qv = csr ? val_b : val_a;
    SpgemmCreateBody body{(cudaStream_t)stream, h, nnz_p, ptr_c};
    const int rc = dispatch_vi(dtype, itype, body);
    if (rc) {
        gsa_spgemm_destroy(h);
        return rc;
    }
    *nnz_c = h->nnz_c;
    *handle = h;
    return GSA_OK;
}

int gsa_spgemm_compute(void *stream, gsa_spgemm *handle, void *idx_c, void *val_c) {
    using namespace gsa;
    if (!handle) return fail(GSA_ERR_INVALID_ARG, "handle is NULL");
    if (handle->nnz_c == 0) return GSA_OK;
    if (!idx_c || !val_c) return fail(GSA_ERR_INVALID_ARG, "output arrays are NULL");
    if (sg_misaligned(idx_c, itype_size(handle->itype)) || sg_misaligned(val_c, dtype_size(handle->dtype)))
        return fail(GSA_ERR_INVALID_ARG, "arrays must be aligned to their element size");
    SpgemmComputeBody body{(cudaStream_t)stream, handle, idx_c, val_c};
    return dispatch_vi(handle->dtype, handle->itype, body);
}

}  // extern "C"
