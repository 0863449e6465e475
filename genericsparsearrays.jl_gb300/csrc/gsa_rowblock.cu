// Row-block gather: C[o, c] = beta*C[o, c] + alpha * sum_j a_j * op(B)(idx_j, c)
// -- kernel_spmatmul_csr_N! (src/matrix_csr/matrix_csr_kernels.jl:1-22) and
// kernel_spmatmul_csc_T! (src/matrix_csc/matrix_csc_kernels.jl:24-45).
//
// Each CTA of 128 threads owns 128 consecutive outer entries (rows) and one group
// of KC right-hand-side columns; each warp owns 32 of the rows.  From the average
// length of its 32 rows a warp picks G lanes per row (1, 2, ..., 32): a thread
// per row for short rows -- plain loads straight from HBM, where neighbouring
// threads read neighbouring entries so a warp's loads share cache lines, and
// tens of thousands of small CTAs keep enough loads in flight to cover DRAM
// latency without staging -- and groups of G lanes reading consecutive entries
// (coalesced) for longer ones, in G passes over the warp's rows.  For SpMM the
// CTAs of one row block and its column groups are numbered consecutively, so
// they run together and share the row block's entries through L2.
//
// Very long rows, with a plan (gsa_plan_create): the plan lists every row of
// more than LONG_LEN entries cut into chunks of CHUNK entries; extra CTAs give
// each chunk to one warp, which stores a partial sum, and the warp that completes
// a row's last chunk adds the row's partials in chunk order and writes the row.
// Without a plan such a row is one group's work like any other.
//
// Every row's summation order is fixed, so results are deterministic.
#include <vector>

#include "gsa_internal.cuh"

namespace gsa {

constexpr int RB_THREADS = 128;
constexpr int RB_WARPS = RB_THREADS / 32;
constexpr int G1_AVG = 6;       // a thread per row while a warp's rows average <= 6 entries
constexpr int LONG_LEN = 512;   // rows longer than this go to a plan's chunks
constexpr int UNROLL = 4;       // entries per lane in flight on the chunk path
constexpr int CHUNK = 512;      // entries per chunk of a planned long row

// acc[c] += sum over j = jb, jb+S, ... < je of conj?(a_j) * op(B)(idx_j, c0 + c), in j order.
template <typename V, typename I, int KC, int S, int U>
__device__ __forceinline__ void accumulate_range(const CompressedArgs<V, I> &a, const DenseIn<V> &B,
                                                 int64_t jb, int64_t je, int64_t c0, int64_t k,
                                                 V (&acc)[KC]) {
    const I *__restrict__ idx = a.idx;
    const V *__restrict__ val = a.val;
    const uint64_t inner = (uint64_t)a.inner_n;
    int64_t j = jb;
    if (U > 1) {
        for (; j + (U - 1) * S < je; j += U * S) {
            int64_t ci[U];
            V av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ci[u] = (int64_t)idx[j + u * S] - a.base;
                av[u] = conj_if(val[j + u * S], a.conjA);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = (uint64_t)ci[u] < inner;
#pragma unroll
                for (int c = 0; c < KC; ++c)
                    if (KC == 1 || c0 + c < k) {
                        const V xv = ok ? B.at(ci[u], c0 + c) : VT<V>::zero();
                        acc[c] = add(acc[c], mul(av[u], xv));
                    }
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

// The plan's view of long rows (device arrays; see gsa_plan).
struct LongRows {
    int64_t nlong, nchunks;
    const int64_t *row;        // nlong: outer index of each long row
    const int32_t *first;      // nlong: its first chunk
    const int32_t *count;      // nlong: its number of chunks
    const int32_t *chunk_slot; // nchunks: the long row (slot) a chunk belongs to
    int *done;                 // nlong * ncg counters, zero before the launch, reset after
    void *partial;             // nchunks * k values
};

// The 32 rows of one warp (lane l owns row row0 + l, entries [b, e)), G lanes per
// row: in each of G passes the warp's 32/G groups take one row each, the group's
// lanes stride the row, a width-G shuffle tree reduces, the group's first lane
// stores.  G = 1 is a thread per row.
template <typename V, typename I, int KC, int G>
__device__ __forceinline__ void warp_rows(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                          const DenseOut<V> &C, int64_t c0, int64_t row0, int64_t b,
                                          int64_t e, int skip) {
    const int lane = threadIdx.x & 31;
    constexpr int RPP = 32 / G;  // rows per pass
#pragma unroll 1
    for (int p = 0; p < G; ++p) {
        const int q = p * RPP + lane / G;
        const int64_t qb = G == 1 ? b : __shfl_sync(0xffffffffu, b, q);
        const int64_t qe = G == 1 ? e : __shfl_sync(0xffffffffu, e, q);
        const int qskip = G == 1 ? skip : __shfl_sync(0xffffffffu, skip, q);
        V acc[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
        accumulate_range<V, I, KC, G, (G == 1 ? 1 : 2)>(a, B, qb + (lane % G), qe, c0, k, acc);
        if (G > 1) {
#pragma unroll
            for (int c = 0; c < KC; ++c) {
#pragma unroll
                for (int m = G / 2; m > 0; m >>= 1) acc[c] = add(acc[c], shfl_xor(acc[c], m, G));
            }
        }
        const int64_t row = row0 + q;
        if (lane % G == 0 && row < a.outer_n && !qskip) {
#pragma unroll
            for (int c = 0; c < KC; ++c)
                if (KC == 1 || c0 + c < k) C.store(row, c0 + c, acc[c]);
        }
    }
}

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS)
rowblock_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t ncg,
                int64_t nrb, LongRows L) {
    const int lane = threadIdx.x & 31;
    // column group fastest; one group (SpMV) needs no division
    const unsigned cta = blockIdx.x;
    const unsigned cg = ncg == 1 ? 0u : cta % (unsigned)ncg;
    const int64_t unit = ncg == 1 ? (int64_t)cta : (int64_t)(cta / (unsigned)ncg);
    const int64_t c0 = (int64_t)cg * KC;

    if (unit >= nrb) {
        // ---- planned long rows: a warp per chunk
        const int64_t chunk = (unit - nrb) * RB_WARPS + (threadIdx.x >> 5);
        if (chunk >= L.nchunks) return;
        const int slot = L.chunk_slot[chunk];
        const int64_t row = L.row[slot];
        const int64_t rb = (int64_t)__ldg(a.ptr + row) - a.base;
        int64_t re = (int64_t)__ldg(a.ptr + row + 1) - a.base;
        re = re > a.nnz ? a.nnz : re;
        const int64_t jb = rb + (chunk - L.first[slot]) * CHUNK;
        const int64_t je = jb + CHUNK < re ? jb + CHUNK : re;
        V acc[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
        accumulate_range<V, I, KC, 32, UNROLL>(a, B, (jb < 0 ? 0 : jb) + lane, je, c0, k, acc);
#pragma unroll
        for (int c = 0; c < KC; ++c) {
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) acc[c] = add(acc[c], shfl_xor(acc[c], m));
        }
        V *part = reinterpret_cast<V *>(L.partial);
        int last = 0;
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < KC; ++c)
                if (c0 + c < k) part[chunk * k + c0 + c] = acc[c];
            __threadfence();
            const int prev = atomicAdd(&L.done[slot * ncg + cg], 1);
            last = prev == L.count[slot] - 1;
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (!last) return;
        // the row's last chunk: add the partials in chunk order
        __threadfence();
        if (lane == 0) {
            const int f = L.first[slot], n = L.count[slot];
#pragma unroll
            for (int c = 0; c < KC; ++c) {
                if (c0 + c >= k) continue;
                V t = VT<V>::zero();
                for (int q = 0; q < n; ++q) t = add(t, ld_coherent(part + (int64_t)(f + q) * k + c0 + c));
                C.store(row, c0 + c, t);
            }
            L.done[slot * ncg + cg] = 0;
        }
        return;
    }

    // ---- this warp's 32 rows, G lanes per row (G from the rows' average length)
    const int64_t row0 = unit * RB_THREADS + (threadIdx.x & ~31);
    const int64_t r = row0 + lane;
    int64_t b = 0, e = 0;
    if (r < a.outer_n) {
        b = (int64_t)__ldg(a.ptr + r) - a.base;
        e = (int64_t)__ldg(a.ptr + r + 1) - a.base;
        b = b < 0 ? 0 : (b > a.nnz ? a.nnz : b);
        e = e < b ? b : (e > a.nnz ? a.nnz : e);
    }
    int skip = 0;
    if (L.nlong > 0 && e - b > LONG_LEN) {  // the plan's chunk CTAs take it
        e = b;
        skip = 1;
    }
    const int64_t total = __shfl_sync(0xffffffffu, e, 31) - __shfl_sync(0xffffffffu, b, 0);
    const int64_t avg = total >> 5;
    if (avg <= G1_AVG) warp_rows<V, I, KC, 1>(a, k, B, C, c0, row0, b, e, skip);
    else if (avg <= 2 * G1_AVG) warp_rows<V, I, KC, 2>(a, k, B, C, c0, row0, b, e, skip);
    else if (avg <= 4 * G1_AVG) warp_rows<V, I, KC, 4>(a, k, B, C, c0, row0, b, e, skip);
    else if (avg <= 8 * G1_AVG) warp_rows<V, I, KC, 8>(a, k, B, C, c0, row0, b, e, skip);
    else if (avg <= 16 * G1_AVG) warp_rows<V, I, KC, 16>(a, k, B, C, c0, row0, b, e, skip);
    else warp_rows<V, I, KC, 32>(a, k, B, C, c0, row0, b, e, skip);
}

// ---------------------------------------------------------------------------
// Plans: which outer entries are long, cut into chunks.

template <typename V, typename I>
int launch_rowblock(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                    DenseOut<V> C, const Plan *plan, void *ws, size_t ws_bytes) {
    if (a.outer_n == 0 || k == 0) return GSA_OK;
    const int64_t nrb = ceil_div(a.outer_n, RB_THREADS);
    // columns a thread accumulates for SpMM: more columns share each entry load, fewer keep
    // registers (and so occupancy) low
    int KC = get_spmm_columns();
    if (KC == 0) KC = sizeof(V) >= 16 ? 2 : 4;
    if (k == 1) KC = 1;
    if (KC > k) KC = k <= 1 ? 1 : (k <= 2 ? 2 : (k <= 4 ? 4 : 8));
    const int64_t ncg = ceil_div(k, KC);
    LongRows L{};
    int64_t units = nrb;
    if (plan && plan->nlong > 0) {
        if (plan->outer_n != a.outer_n || plan->nnz != a.nnz)
            return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
        const size_t need = rowblock_workspace_size(plan, sizeof(V), k);
        if (ws_bytes < need) return fail(GSA_ERR_INVALID_ARG, "rowblock workspace too small");
        Carver cv(ws);
        int *done = cv.take<int>((size_t)(plan->nlong * ncg));
        void *partial = cv.take<V>((size_t)(plan->nchunks * k));
        int rc = check_cuda(cudaMemsetAsync(done, 0, sizeof(int) * plan->nlong * ncg, s), "plan counters");
        if (rc) return rc;
        L = LongRows{plan->nlong, plan->nchunks, plan->row, plan->first, plan->count, plan->chunk_slot,
                     done, partial};
        units += ceil_div(plan->nchunks, RB_WARPS);
    }
    const int64_t blocks = units * ncg;
    if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many rows");
    timer_before(s);
    if (KC == 1) rowblock_kernel<V, I, 1><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else if (KC == 2) rowblock_kernel<V, I, 2><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else if (KC == 4) rowblock_kernel<V, I, 4><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else rowblock_kernel<V, I, 8><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "rowblock_kernel");
}

static int g_spmm_columns = 0;  // 0: by value size
void set_spmm_columns(int c) { g_spmm_columns = c; }
int get_spmm_columns() { return g_spmm_columns; }

size_t rowblock_workspace_size(const Plan *plan, size_t vsize, int64_t k) {
    if (!plan || plan->nlong == 0 || k == 0) return 0;
    const int64_t ncg = k;  // an upper bound on the column groups of any KC
    Carver cv(nullptr);
    cv.take<int>((size_t)(plan->nlong * ncg));
    cv.take<unsigned char>((size_t)(plan->nchunks * k) * vsize + 16);
    return align_up(cv.off, 256);
}

template <typename I>
static int build_plan(cudaStream_t s, int64_t outer_n, int64_t nnz, const I *ptr, int base, Plan *p) {
    std::vector<I> h((size_t)outer_n + 1);
    int rc = check_cuda(cudaMemcpyAsync(h.data(), ptr, sizeof(I) * (outer_n + 1), cudaMemcpyDeviceToHost, s),
                        "plan: pointer copy");
    if (rc) return rc;
    rc = check_cuda(cudaStreamSynchronize(s), "plan: sync");
    if (rc) return rc;
    std::vector<int64_t> row;
    std::vector<int32_t> first, count, slot;
    int64_t maxlen = 0;
    for (int64_t r = 0; r < outer_n; ++r) {
        int64_t b = (int64_t)h[r] - base, e = (int64_t)h[r + 1] - base;
        b = b < 0 ? 0 : (b > nnz ? nnz : b);
        e = e < b ? b : (e > nnz ? nnz : e);
        const int64_t len = e - b;
        maxlen = len > maxlen ? len : maxlen;
        if (len <= LONG_LEN) continue;
        const int64_t nch = ceil_div(len, CHUNK);
        if ((int64_t)slot.size() + nch > 0x7fffffffLL)
            return fail(GSA_ERR_UNSUPPORTED, "plan: too many chunks");
        row.push_back(r);
        first.push_back((int32_t)slot.size());
        count.push_back((int32_t)nch);
        for (int64_t q = 0; q < nch; ++q) slot.push_back((int32_t)(row.size() - 1));
    }
    p->outer_n = outer_n;
    p->nnz = nnz;
    p->max_len = maxlen;
    p->nlong = (int64_t)row.size();
    p->nchunks = (int64_t)slot.size();
    if (p->nlong == 0) return GSA_OK;
    size_t bytes = align_up(row.size() * 8, 256) + align_up(first.size() * 4, 256) +
                   align_up(count.size() * 4, 256) + align_up(slot.size() * 4, 256);
    rc = check_cuda(cudaMalloc(&p->mem, bytes), "plan: device memory");
    if (rc) return rc;
    Carver cv(p->mem);
    int64_t *d_row = cv.take<int64_t>(row.size());
    int32_t *d_first = cv.take<int32_t>(first.size());
    int32_t *d_count = cv.take<int32_t>(count.size());
    int32_t *d_slot = cv.take<int32_t>(slot.size());
    rc = check_cuda(cudaMemcpy(d_row, row.data(), row.size() * 8, cudaMemcpyHostToDevice), "plan: rows");
    if (!rc) rc = check_cuda(cudaMemcpy(d_first, first.data(), first.size() * 4, cudaMemcpyHostToDevice), "plan: first");
    if (!rc) rc = check_cuda(cudaMemcpy(d_count, count.data(), count.size() * 4, cudaMemcpyHostToDevice), "plan: count");
    if (!rc) rc = check_cuda(cudaMemcpy(d_slot, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice), "plan: chunks");
    if (rc) return rc;
    p->row = d_row;
    p->first = d_first;
    p->count = d_count;
    p->chunk_slot = d_slot;
    return GSA_OK;
}

int plan_create(cudaStream_t s, int itype, int64_t outer_n, int64_t nnz, const void *ptr, int base, Plan *p) {
    if (itype == GSA_IDX32) return build_plan<int32_t>(s, outer_n, nnz, (const int32_t *)ptr, base, p);
    return build_plan<int64_t>(s, outer_n, nnz, (const int64_t *)ptr, base, p);
}

#define GSA_INST_RB(V, I)                                                                       \
    template int launch_rowblock<V, I>(cudaStream_t, const CompressedArgs<V, I> &, int64_t,     \
                                       DenseIn<V>, DenseOut<V>, const Plan *, void *, size_t);
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
