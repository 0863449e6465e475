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
// Longer rows, with a plan (gsa_plan_create): the plan lists every row of more
// than CHUNK entries and every row of more than PLAN_LEN entries that is over 4x
// its warp's average, cut into chunks of CHUNK entries; extra CTAs give each
// chunk to one warp (32 lanes, UNROLL loads each in flight).  A row of one chunk
// is summed and stored by its warp; for a longer one each warp stores a partial
// sum, and the warp that completes the row's last chunk adds the partials in chunk
// order and writes the row.  A warp of short rows thus never waits on a long one.
// Without a plan such a row is one group's work like any other.
//
// Every row's summation order is fixed, so results are deterministic.
#include <vector>

#include "gsa_rows.cuh"

namespace gsa {

// Resident CTAs per SM the compiler must allow: the one-column kernels of 4- and 8-byte
// values are latency-bound gathers whose speed follows the warps in flight, so they are
// held to 32 registers (16 CTAs of 128 threads, every warp slot of the SM).  0 leaves
// the register count to the compiler.
#ifndef GSA_RB_MIN_BLOCKS
#define GSA_RB_MIN_BLOCKS 16
#endif
template <typename V, int KC> constexpr int rb_min_blocks() { return KC * sizeof(V) <= 8 ? GSA_RB_MIN_BLOCKS : 0; }

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS, rb_min_blocks<V, KC>())
rowblock_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t ncg,
                int64_t nrb, PlanRows L) {
    const int lane = threadIdx.x & 31;
    // column group fastest; one group (SpMV) needs no division
    const unsigned cta = blockIdx.x;
    const unsigned cg = ncg == 1 ? 0u : cta % (unsigned)ncg;
    const int64_t unit = ncg == 1 ? (int64_t)cta : (int64_t)(cta / (unsigned)ncg);
    const int64_t c0 = (int64_t)cg * KC;

    if (unit >= nrb) {
        // ---- planned rows: a warp per chunk of up to CHUNK entries
        using O = Off<I>;
        const int64_t chunk = (unit - nrb) * RB_WARPS + (threadIdx.x >> 5);
        if (chunk >= L.nchunks) return;
        const int slot = L.chunk_slot[chunk];
        const int64_t row = L.row[slot];
        const int nch = L.count[slot];
        const O nz = (O)a.nnz, base = (O)a.base;
        O rb = (O)__ldg(a.ptr + row) - base;
        O re = (O)__ldg(a.ptr + row + 1) - base;
        rb = rb < nz ? rb : nz;
        re = re < nz ? re : nz;
        const O jb = rb + (O)(chunk - L.first[slot]) * (O)CHUNK;
        const O je = jb < re && re - jb > (O)CHUNK ? jb + (O)CHUNK : re;
        V acc[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
        if (jb < je) accumulate_range<V, I, KC, 32, UNROLL>(a, B, jb + (O)lane, je, c0, k, acc);
#pragma unroll
        for (int c = 0; c < KC; ++c) {
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) acc[c] = add(acc[c], shfl_xor(acc[c], m));
        }
        if (nch == 1) {  // the whole row: store it
            if (lane == 0) {
#pragma unroll
                for (int c = 0; c < KC; ++c)
                    if (c0 + c < k) C.store(row, c0 + c, acc[c]);
            }
            return;
        }
        V *part = reinterpret_cast<V *>(L.partial);
        int last = 0;
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < KC; ++c)
                if (c0 + c < k) part[chunk * k + c0 + c] = acc[c];
            __threadfence();
            const int prev = atomicAdd(&L.done[slot * ncg + cg], 1);
            last = prev == nch - 1;
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (!last) return;
        // the row's last chunk: add the partials in chunk order
        __threadfence();
        if (lane == 0) {
            const int f = L.first[slot];
#pragma unroll
            for (int c = 0; c < KC; ++c) {
                if (c0 + c >= k) continue;
                V t = VT<V>::zero();
                for (int q = 0; q < nch; ++q) t = add(t, ld_coherent(part + (int64_t)(f + q) * k + c0 + c));
                C.store(row, c0 + c, t);
            }
            L.done[slot * ncg + cg] = 0;
        }
        return;
    }

    // ---- this warp's 32 rows
    warp_unit<V, I, KC>(a, k, B, C, c0, unit * RB_THREADS + (threadIdx.x & ~31), L.skip_mask);
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
    PlanRows L{};
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
        L = PlanRows{plan->nlong, plan->nchunks, plan->row, plan->first, plan->count, plan->chunk_slot,
                     plan->skip_mask, done, partial};
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
    std::vector<int64_t> len((size_t)outer_n);
    int64_t maxlen = 0;
    for (int64_t r = 0; r < outer_n; ++r) {
        int64_t b = (int64_t)h[r] - base, e = (int64_t)h[r + 1] - base;
        b = b < 0 ? 0 : (b > nnz ? nnz : b);
        e = e < b ? b : (e > nnz ? nnz : e);
        len[r] = e - b;
        maxlen = len[r] > maxlen ? len[r] : maxlen;
    }
    // A row goes to the plan when it is longer than CHUNK, or longer than PLAN_LEN and
    // more than 4x the average of its warp's 32 rows (it would hold the warp's other
    // rows back).  Rows of even length stay in their warps, G lanes per row.
    std::vector<int64_t> row;
    std::vector<int32_t> first, count, slot;
    std::vector<uint32_t> mask((size_t)ceil_div(outer_n, 32), 0u);
    for (int64_t w0 = 0; w0 < outer_n; w0 += 32) {
        const int64_t w1 = w0 + 32 < outer_n ? w0 + 32 : outer_n;
        int64_t sum = 0;
        for (int64_t r = w0; r < w1; ++r) sum += len[r];
        for (int64_t r = w0; r < w1; ++r) {
            if (len[r] <= PLAN_LEN || (len[r] <= CHUNK && 8 * len[r] <= sum)) continue;
            const int64_t nch = ceil_div(len[r], CHUNK);
            if ((int64_t)slot.size() + nch > 0x7fffffffLL)
                return fail(GSA_ERR_UNSUPPORTED, "plan: too many chunks");
            mask[(size_t)(w0 >> 5)] |= 1u << (r - w0);
            row.push_back(r);
            first.push_back((int32_t)slot.size());
            count.push_back((int32_t)nch);
            for (int64_t q = 0; q < nch; ++q) slot.push_back((int32_t)(row.size() - 1));
        }
    }
    p->outer_n = outer_n;
    p->nnz = nnz;
    p->max_len = maxlen;
    p->nlong = (int64_t)row.size();
    p->nchunks = (int64_t)slot.size();
    if (p->nlong == 0) return GSA_OK;
    size_t bytes = align_up(row.size() * 8, 256) + align_up(first.size() * 4, 256) +
                   align_up(count.size() * 4, 256) + align_up(slot.size() * 4, 256) +
                   align_up(mask.size() * 4, 256);
    rc = check_cuda(cudaMalloc(&p->mem, bytes), "plan: device memory");
    if (rc) return rc;
    Carver cv(p->mem);
    int64_t *d_row = cv.take<int64_t>(row.size());
    int32_t *d_first = cv.take<int32_t>(first.size());
    int32_t *d_count = cv.take<int32_t>(count.size());
    int32_t *d_slot = cv.take<int32_t>(slot.size());
    uint32_t *d_mask = cv.take<uint32_t>(mask.size());
    rc = check_cuda(cudaMemcpy(d_row, row.data(), row.size() * 8, cudaMemcpyHostToDevice), "plan: rows");
    if (!rc) rc = check_cuda(cudaMemcpy(d_first, first.data(), first.size() * 4, cudaMemcpyHostToDevice), "plan: first");
    if (!rc) rc = check_cuda(cudaMemcpy(d_count, count.data(), count.size() * 4, cudaMemcpyHostToDevice), "plan: count");
    if (!rc) rc = check_cuda(cudaMemcpy(d_slot, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice), "plan: chunks");
    if (!rc) rc = check_cuda(cudaMemcpy(d_mask, mask.data(), mask.size() * 4, cudaMemcpyHostToDevice), "plan: mask");
    if (rc) return rc;
    p->row = d_row;
    p->first = d_first;
    p->count = d_count;
    p->chunk_slot = d_slot;
    p->skip_mask = d_mask;
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
