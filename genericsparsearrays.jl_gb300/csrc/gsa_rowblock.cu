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
#include <algorithm>
#include <atomic>
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
// The bin order's ComplexF64 SpMV is held to 8 resident CTAs, which lets the compiler keep 64
// registers (48 without the bound) and more loads in flight: power-law n = 10^6 160 us against
// 170 us on one GB300 (12 CTAs at 40 registers: 177 us, 10 at 48: 167 us, 7 at 72: 163 us, 6 at
// 74: 169 us, 5 at 88: 178 us); the grouped kernel gained nothing from the same bounds.
#ifndef GSA_BINNED_C64_MIN_BLOCKS
#define GSA_BINNED_C64_MIN_BLOCKS 8
#endif
template <typename V, int KC> constexpr int binned_min_blocks() {
    return std::is_same<V, cf64>::value && KC == 1 ? GSA_BINNED_C64_MIN_BLOCKS : rb_min_blocks<V, KC>();
}

// The bin order pays where the FP64 pipe binds: ComplexF64 products (four FMAs per entry)
// and Float64 products with several right-hand sides (one FMA per entry and column); a
// Float64 SpMV is HBM-bound, and there the scattered rows cost more traffic than idle lanes
// cost time (Poisson(10), 2M rows: 112 us natural vs 226 us binned).
template <typename V> constexpr bool bins_possible() {
    return std::is_same<V, cf64>::value || std::is_same<V, double>::value;
}
template <typename V> inline bool bins_pay(int64_t k) {
    return std::is_same<V, cf64>::value || (std::is_same<V, double>::value && k > 1);
}

// One warp sums chunk `chunk` of a chunked row (entries [jb, je), 32 lanes, UNROLL loads
// each in flight).  A row of one chunk is stored at once; otherwise the warp stores its
// partial sum, and the warp that completes the row's last chunk adds the partials in
// chunk order and writes the row.
template <typename V, typename I, int KC>
__device__ __forceinline__ void chunk_unit(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                           const DenseOut<V> &C, int64_t c0, unsigned cg, int64_t ncg,
                                           int64_t chunk, const PlanRows &L) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
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
}

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS, rb_min_blocks<V, KC>())
rowblock_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t ncg,
                int64_t nrb, PlanRows L) {
    // column group fastest; one group (SpMV) needs no division
    const unsigned cta = blockIdx.x;
    const unsigned cg = ncg == 1 ? 0u : cta % (unsigned)ncg;
    const int64_t unit = ncg == 1 ? (int64_t)cta : (int64_t)(cta / (unsigned)ncg);
    const int64_t c0 = (int64_t)cg * KC;
    if (unit >= nrb) {  // chunked rows: a warp per chunk
        chunk_unit<V, I, KC>(a, k, B, C, c0, cg, ncg, (unit - nrb) * RB_WARPS + (threadIdx.x >> 5), L);
        return;
    }
    // ---- this warp's 32 rows
    warp_unit<V, I, KC>(a, k, B, C, c0, unit * RB_THREADS + (threadIdx.x & ~31), L.skip_mask);
}

// ---------------------------------------------------------------------------
// Staged rows (GSA_TUNE_STAGE_ROWS = 1; one right-hand side, Float32 or Float64 values, Int32
// indices): the entries of a warp's 32 thread-per-row rows are one contiguous span, which the
// warp copies into shared memory with 16-byte loads -- a lane moves whole 16-byte pieces of
// idx and val, two or three warp instructions where the direct path issues one scalar load
// per entry and lane -- before each lane sums its own row from shared memory.  Warps whose
// rows take several lanes, spans longer than STAGE_CAP entries, spans whose 16-byte pieces
// would pass the end of the arrays and arrays that are not 16-byte aligned take the direct
// path of rowblock_kernel.  Each row is summed in the same order as there (bit-identical).
constexpr int STAGE_CAP = 256;

template <typename V> constexpr bool stage_rows_type() {
    return std::is_same<V, float>::value || std::is_same<V, double>::value;
}

// 12 resident CTAs of 128 threads: 40 registers, and 96 KB (Float32) or 144 KB (Float64) of
// staging per SM
template <typename V, typename I>
__global__ void __launch_bounds__(RB_THREADS, 12)
rowblock_staged_kernel(CompressedArgs<V, I> a, DenseIn<V> B, DenseOut<V> C, int64_t nrb, PlanRows L) {
    static_assert(sizeof(I) == 4, "staged rows take 32-bit offsets");
    constexpr int PIECE = 4;  // entries per 16 bytes of indices (and the unit of the span's ends)
    __shared__ __align__(16) I s_idx[RB_WARPS][STAGE_CAP];
    __shared__ __align__(16) V s_val[RB_WARPS][STAGE_CAP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t unit = blockIdx.x;
    if (unit >= nrb) {  // chunked rows: a warp per chunk
        chunk_unit<V, I, 1>(a, 1, B, C, 0, 0u, 1, (unit - nrb) * RB_WARPS + w, L);
        return;
    }
    const int64_t row0 = unit * RB_THREADS + (threadIdx.x & ~31);
    if (row0 >= a.outer_n) return;  // a warp past the last row (uniform: the whole warp leaves)
    uint32_t b, e;
    int skip;
    const int64_t avg = warp_extent(a, row0, L.skip_mask, b, e, skip);
    // lane 0's row exists, so the span [S, E) covers at least one row: S <= b_0 <= e_0 <= E
    const bool valid = row0 + lane < a.outer_n;
    const uint32_t S = __reduce_min_sync(0xffffffffu, valid ? b : 0xffffffffu) & ~(uint32_t)(PIECE - 1);
    const uint32_t E = __reduce_max_sync(0xffffffffu, valid ? e : 0u);
    const uint32_t T = (E + PIECE - 1) & ~(uint32_t)(PIECE - 1);
    if (avg > G1_AVG || T < S || T - S > (uint32_t)STAGE_CAP || (int64_t)T > a.nnz) {
        dispatch_lanes(avg, G1_AVG, [&](auto g) {
            warp_rows<V, I, 1, decltype(g)::value>(a, 1, B, C, 0, row0, b, e, skip);
        });
        return;
    }
    // the span [S, T) in 16-byte pieces
    const int4 *gi = reinterpret_cast<const int4 *>(a.idx + S);
    int4 *si = reinterpret_cast<int4 *>(&s_idx[w][0]);
    for (uint32_t q = lane; q < (T - S) / PIECE; q += 32) si[q] = __ldcs(gi + q);
    constexpr int VPIECE = 16 / sizeof(V);
    using V4 = typename std::conditional<sizeof(V) == 4, float4, double2>::type;
    const V4 *gv = reinterpret_cast<const V4 *>(a.val + S);
    V4 *sv = reinterpret_cast<V4 *>(&s_val[w][0]);
    for (uint32_t q = lane; q < (T - S) / VPIECE; q += 32) sv[q] = __ldcs(gv + q);
    __syncwarp();
    const uint32_t inner = a.inner_n < 0xffffffffLL ? (uint32_t)a.inner_n : 0xffffffffu;
    const uint32_t base = (uint32_t)a.base;
    V acc = VT<V>::zero();
    uint32_t j = b - S;
    const uint32_t je = e - S;
    for (; j + 3 < je; j += 4) {  // four gathers in flight
        uint32_t ci[4];
        V av[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            ci[u] = (uint32_t)s_idx[w][j + u] - base;
            av[u] = s_val[w][j + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = mac(acc, av[u], ci[u] < inner ? B.at((int64_t)ci[u], 0) : VT<V>::zero());
    }
    for (; j < je; ++j) {
        const uint32_t c1 = (uint32_t)s_idx[w][j] - base;
        acc = mac(acc, s_val[w][j], c1 < inner ? B.at((int64_t)c1, 0) : VT<V>::zero());
    }
    if (valid && !skip) C.store(row0 + lane, 0, acc);
}

// Vector rows (GSA_TUNE_STAGE_ROWS = 2; same types as the staged rows): each lane of a
// thread-per-row warp reads its own row's indices and values in aligned 16-byte pieces
// straight into registers -- one 16-byte index load and one or two value loads per four
// entries, where the direct path issues a scalar load per entry and array -- and multiplies the
// entries of each piece that lie in its row, in order (bit-identical to the direct path).  A
// lane whose last piece would pass the end of the arrays uses scalar loads.
template <typename V, typename I>
__global__ void __launch_bounds__(RB_THREADS, rb_min_blocks<V, 1>())
rowblock_vec_kernel(CompressedArgs<V, I> a, DenseIn<V> B, DenseOut<V> C, int64_t nrb, PlanRows L) {
    static_assert(sizeof(I) == 4, "vector rows take 32-bit offsets");
    const int w = threadIdx.x >> 5;
    const int64_t unit = blockIdx.x;
    if (unit >= nrb) {  // chunked rows: a warp per chunk
        chunk_unit<V, I, 1>(a, 1, B, C, 0, 0u, 1, (unit - nrb) * RB_WARPS + w, L);
        return;
    }
    const int64_t row0 = unit * RB_THREADS + (threadIdx.x & ~31);
    if (row0 >= a.outer_n) return;  // a warp past the last row (uniform)
    uint32_t b, e;
    int skip;
    const int64_t avg = warp_extent(a, row0, L.skip_mask, b, e, skip);
    if (avg > G1_AVG) {
        dispatch_lanes(avg, G1_AVG, [&](auto g) {
            warp_rows<V, I, 1, decltype(g)::value>(a, 1, B, C, 0, row0, b, e, skip);
        });
        return;
    }
    const int lane = threadIdx.x & 31;
    const uint32_t inner = a.inner_n < 0xffffffffLL ? (uint32_t)a.inner_n : 0xffffffffu;
    const uint32_t base = (uint32_t)a.base;
    V acc = VT<V>::zero();
    if ((int64_t)((e + 3u) & ~3u) <= a.nnz) {
#pragma unroll 2
        for (uint32_t c = b & ~3u; c < e; c += 4) {
            const int4 iv = __ldcs(reinterpret_cast<const int4 *>(a.idx + c));
            V v[4];
            if constexpr (sizeof(V) == 4) {
                const float4 f = __ldcs(reinterpret_cast<const float4 *>(a.val + c));
                v[0] = f.x; v[1] = f.y; v[2] = f.z; v[3] = f.w;
            } else {
                const double2 d0 = __ldcs(reinterpret_cast<const double2 *>(a.val + c));
                const double2 d1 = __ldcs(reinterpret_cast<const double2 *>(a.val + c + 2));
                v[0] = d0.x; v[1] = d0.y; v[2] = d1.x; v[3] = d1.y;
            }
            const uint32_t ci[4] = {(uint32_t)iv.x - base, (uint32_t)iv.y - base, (uint32_t)iv.z - base,
                                    (uint32_t)iv.w - base};
            V x[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const bool in = c + t >= b && c + t < e;
                x[t] = in && ci[t] < inner ? B.at((int64_t)ci[t], 0) : VT<V>::zero();
            }
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (c + t >= b && c + t < e) acc = mac(acc, v[t], x[t]);
        }
    } else {
        for (uint32_t j = b; j < e; ++j) {
            const uint32_t c1 = (uint32_t)a.idx[j] - base;
            acc = mac(acc, a.val[j], c1 < inner ? B.at((int64_t)c1, 0) : VT<V>::zero());
        }
    }
    if (row0 + lane < a.outer_n && !skip) C.store(row0 + lane, 0, acc);
}

static std::atomic<int> g_x_pairs{1};
void set_x_pairs(int v) { g_x_pairs.store(v, std::memory_order_relaxed); }
int get_x_pairs() { return g_x_pairs.load(std::memory_order_relaxed); }

static std::atomic<int> g_stage_rows{0};
void set_stage_rows(int v) { g_stage_rows.store(v, std::memory_order_relaxed); }
int get_stage_rows() { return g_stage_rows.load(std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// Bin order: within each segment of BIN_SEGMENT rows the plan sorts the rows by the
// multiply-adds each of their lanes does (rows up to 32 entries with a lane each, longer
// ones with G = 2, 4, 8 or 16 lanes, each lane 17 to 32 entries) and warp w of the order
// takes 32 / G consecutive rows of one lanes-per-row class of one segment.  The lanes of a
// warp then do the same number of multiply-adds, or one apart: FP64 products on GB300 are
// bound by the FP64 pipe, which counts a warp instruction whole however few of its lanes
// are active.  A segment's rows are read close together in time, so the sectors that
// neighbouring rows share are still in L2 when the second of them is read.

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS, binned_min_blocks<V, KC>())
binned_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t ncg, gsa_bin_order bv,
              PlanRows L) {
    const unsigned cta = blockIdx.x;
    const unsigned cg = ncg == 1 ? 0u : cta % (unsigned)ncg;
    const int64_t unit = ncg == 1 ? (int64_t)cta : (int64_t)(cta / (unsigned)ncg);
    const int64_t c0 = (int64_t)cg * KC;
    const int64_t w = unit * RB_WARPS + (threadIdx.x >> 5);
    if (w >= bv.nwarps) {  // chunked rows
        chunk_unit<V, I, KC>(a, k, B, C, c0, cg, ncg, w - bv.nwarps, L);
        return;
    }
    binned_warp<V, I, KC>(a, k, B, C, c0, w, bv);
}

template <typename V, typename I>
int launch_rowblock(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                    DenseOut<V> C, const Plan *plan, void *ws, size_t ws_bytes) {
    if (a.outer_n == 0 || k == 0) return GSA_OK;
    const int64_t nrb = ceil_div(a.outer_n, RB_THREADS);
    // columns a thread accumulates for SpMM: more columns share each entry load, fewer keep
    // registers (and so occupancy) low
    // (measured defaults: with a column-major B each column is its own gather, and the
    // FP64-bound 8-byte types do best with 2 columns, 16-byte ones with 4; with a row-major
    // B an entry's values share cache lines and a thread reads them in 16-byte pieces: 8 columns
    // (Float64 SpMM of the served mix's matrices, n = 10^6, k = 16: 871 us with 8 against 982 us
    // with 4); 4-byte values take 4)
    int KC = get_spmm_columns();
    if (KC == 0) {
        const bool rowmajor = B.cs == 1 && B.rs > 1;
        KC = sizeof(V) >= 16 ? (rowmajor ? 8 : 4) : (sizeof(V) == 8 ? (rowmajor ? 8 : 2) : 4);
    }
    if (k == 1) KC = 1;
    if (KC > k) KC = k <= 1 ? 1 : (k <= 2 ? 2 : (k <= 4 ? 4 : 8));
    const int64_t ncg = ceil_div(k, KC);
    B.pairs = KC >= 2 && get_x_pairs() && pairs_ok(B);
    if (plan && (plan->outer_n != a.outer_n || plan->nnz != a.nnz))
        return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
    // plan order 0: the bin order where it pays; 1: natural always; 2: the bin order for every
    // FP64 product whose plan has one
    const int order = get_plan_natural();
    const bool binned = plan && plan->nbin_warps > 0 && order != 1 && (order == 2 || bins_pay<V>(k));
    PlanRows L{};
    int64_t chunk_warps = 0;
    const gsa_chunk_set *cs = plan ? (binned ? &plan->bin : &plan->nat) : nullptr;
    if (cs && cs->nlong > 0) {
        const size_t need = rowblock_workspace_size(plan, sizeof(V), k);
        if (ws_bytes < need) return fail(GSA_ERR_INVALID_ARG, "rowblock workspace too small");
        Carver cv(ws);
        int *done = cv.take<int>((size_t)(cs->nlong * ncg));
        void *partial = cv.take<V>((size_t)(cs->nchunks * k));
        int rc = check_cuda(cudaMemsetAsync(done, 0, sizeof(int) * cs->nlong * ncg, s), "plan counters");
        if (rc) return rc;
        L = plan_rows(*cs);
        L.done = done;
        L.partial = partial;
        chunk_warps = cs->nchunks;
    }
    const int64_t units = binned ? ceil_div(plan->nbin_warps + chunk_warps, RB_WARPS)
                                 : nrb + ceil_div(chunk_warps, RB_WARPS);
    const int64_t blocks = units * ncg;
    if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many rows");
    timer_before(s);
    if constexpr (bins_possible<V>()) {  // the only types a bin order runs for: no other instances
        if (binned) {
            const gsa_bin_order bv = plan->order;
            if (KC == 1) binned_kernel<V, I, 1><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, bv, L);
            else if (KC == 2) binned_kernel<V, I, 2><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, bv, L);
            else if (KC == 4) binned_kernel<V, I, 4><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, bv, L);
            else binned_kernel<V, I, 8><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, bv, L);
            timer_after(s);
            return check_cuda(cudaGetLastError(), "binned_kernel");
        }
    }
    if constexpr (stage_rows_type<V>() && sizeof(I) == 4) {
        const bool aligned = ((uintptr_t)a.idx % 16 == 0) && ((uintptr_t)a.val % 16 == 0);
        if (KC == 1 && get_stage_rows() == 1 && aligned) {
            rowblock_staged_kernel<V, I><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, B, C, nrb, L);
            timer_after(s);
            return check_cuda(cudaGetLastError(), "rowblock_staged_kernel");
        }
        if (KC == 1 && get_stage_rows() == 2 && aligned) {
            rowblock_vec_kernel<V, I><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, B, C, nrb, L);
            timer_after(s);
            return check_cuda(cudaGetLastError(), "rowblock_vec_kernel");
        }
    }
    if (KC == 1) rowblock_kernel<V, I, 1><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else if (KC == 2) rowblock_kernel<V, I, 2><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else if (KC == 4) rowblock_kernel<V, I, 4><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    else rowblock_kernel<V, I, 8><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, L);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "rowblock_kernel");
}

// Process-wide tuning knobs: atomics, since any host thread may set them while others launch.
static std::atomic<int> g_spmm_columns{0};  // 0: by value size
void set_spmm_columns(int c) { g_spmm_columns.store(c, std::memory_order_relaxed); }
int get_spmm_columns() { return g_spmm_columns.load(std::memory_order_relaxed); }
static std::atomic<int> g_plan_order{0};    // 0: the plan's choice, 1: natural order always
void set_plan_natural(int v) { g_plan_order.store(v, std::memory_order_relaxed); }
int get_plan_natural() { return g_plan_order.load(std::memory_order_relaxed); }

size_t rowblock_workspace_size(const Plan *plan, size_t vsize, int64_t k) {
    if (!plan || k == 0) return 0;
    // enough for either chunk set; ncg <= k for any KC
    const int64_t nlong = plan->nat.nlong > plan->bin.nlong ? plan->nat.nlong : plan->bin.nlong;
    const int64_t nchunks = plan->nat.nchunks > plan->bin.nchunks ? plan->nat.nchunks : plan->bin.nchunks;
    if (nlong == 0) return 0;
    Carver cv(nullptr);
    cv.take<int>((size_t)(nlong * k));
    cv.take<unsigned char>((size_t)(nchunks * k) * vsize + 16);
    return align_up(cv.off, 256);
}

// ---------------------------------------------------------------------------
// Plans.

// Bin of a row of len <= CHUNK entries and its lanes per row: rows of equal length up to
// 32 (a lane each), then for 32 < len <= 512 the G = 2, 4, 8 or 16 lanes with 16 <
// ceil(len / G) <= 32 and one bin per value of ceil(len / G): every lane of a warp does
// the same number of multiply-adds, 17 to 32, before the width-G reduction.
constexpr int NBINS = 97;
constexpr int64_t BIN_SEGMENT = 32768;  // rows per segment of the bin order
static int bin_of(int64_t len) {
    if (len <= 32) return (int)len;
    int lg = 1;
    while (((int64_t)32 << lg) < len) ++lg;  // G = 2^lg lanes: 32 * G >= len
    const int64_t q = (len + ((int64_t)1 << lg) - 1) >> lg;  // 17 .. 32
    return 33 + (lg - 1) * 16 + (int)(q - 17);
}
static int bin_lanes(int b) { return b <= 32 ? 1 : 1 << (1 + (b - 33) / 16); }

// Lane utilisation of the natural order: the fraction of lane-iterations that do a
// multiply-add when a warp of 32 rows runs G lanes per row (G from the rows' average, as
// warp_extent and dispatch_lanes pick it) and each pass lasts as long as its longest row.
static double natural_utilisation(const std::vector<int64_t> &len, const std::vector<uint32_t> &mask) {
    double busy = 0, held = 0;
    const int64_t n = (int64_t)len.size();
    for (int64_t w0 = 0; w0 < n; w0 += 32) {
        const int64_t w1 = w0 + 32 < n ? w0 + 32 : n;
        int64_t l[32] = {0};
        int64_t total = 0;
        for (int64_t r = w0; r < w1; ++r) {
            const bool skip = (mask[(size_t)(w0 >> 5)] >> (r - w0)) & 1u;
            l[r - w0] = skip ? 0 : len[r];
            total += l[r - w0];
        }
        const int64_t avg = total >> 5;
        int G = 1;
        while (G < 32 && avg > (int64_t)G * G1_AVG) G <<= 1;
        for (int p = 0; p < G; ++p) {
            int64_t longest = 0;
            for (int q = p * (32 / G); q < (p + 1) * (32 / G); ++q)
                longest = l[q] > longest ? l[q] : longest;
            held += 32.0 * (double)ceil_div(longest, G);
        }
        busy += (double)total;
    }
    return held > 0 ? busy / held : 1.0;
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
    // Natural order: a row goes to chunks when it is longer than CHUNK, or longer than
    // PLAN_LEN and more than 4x the average of its warp's 32 rows (it would hold the
    // warp's other rows back).  Bin order: only rows longer than CHUNK are chunked.
    std::vector<uint32_t> mask_nat((size_t)ceil_div(outer_n, 32), 0u), mask_bin(mask_nat.size(), 0u);
    for (int64_t w0 = 0; w0 < outer_n; w0 += 32) {
        const int64_t w1 = w0 + 32 < outer_n ? w0 + 32 : outer_n;
        int64_t sum = 0;
        for (int64_t r = w0; r < w1; ++r) sum += len[r];
        for (int64_t r = w0; r < w1; ++r) {
            if (len[r] > CHUNK) mask_bin[(size_t)(w0 >> 5)] |= 1u << (r - w0);
            if (len[r] > CHUNK || (len[r] > PLAN_LEN && 8 * len[r] > sum))
                mask_nat[(size_t)(w0 >> 5)] |= 1u << (r - w0);
        }
    }
    // bin order when the natural one would leave over a tenth of the lanes idle (only
    // FP64-bound products use it, where every idle lane is lost FP64 time)
    const bool binned = outer_n >= 32 && outer_n <= 0x7fffffffLL && natural_utilisation(len, mask_nat) < 0.9;
    struct HostSet {
        std::vector<int64_t> row;
        std::vector<int32_t> first, count, slot;
    } hs[2];
    for (int t = 0; t < (binned ? 2 : 1); ++t) {
        const std::vector<uint32_t> &mask = t == 0 ? mask_nat : mask_bin;
        HostSet &h2 = hs[t];
        for (int64_t r = 0; r < outer_n; ++r) {
            if (!((mask[(size_t)(r >> 5)] >> (r & 31)) & 1u)) continue;
            const int64_t nch = ceil_div(len[r], CHUNK);
            if ((int64_t)h2.slot.size() + nch > 0x7fffffffLL)
                return fail(GSA_ERR_UNSUPPORTED, "plan: too many chunks");
            h2.row.push_back(r);
            h2.first.push_back((int32_t)h2.slot.size());
            h2.count.push_back((int32_t)nch);
            for (int64_t q = 0; q < nch; ++q) h2.slot.push_back((int32_t)(h2.row.size() - 1));
        }
    }
    std::vector<int32_t> perm, warp_group;
    std::vector<int64_t> groups;
    if (binned) {  // per segment, a counting sort of the unchunked rows by bin, stable
        std::vector<int64_t> cnt(NBINS + 1);
        for (int64_t s0 = 0; s0 < outer_n; s0 += BIN_SEGMENT) {
            const int64_t s1 = s0 + BIN_SEGMENT < outer_n ? s0 + BIN_SEGMENT : outer_n;
            std::fill(cnt.begin(), cnt.end(), 0);
            for (int64_t r = s0; r < s1; ++r)
                if (len[r] <= CHUNK) ++cnt[(size_t)bin_of(len[r]) + 1];
            for (int b = 0; b < NBINS; ++b) cnt[(size_t)b + 1] += cnt[(size_t)b];
            const int64_t base_pos = (int64_t)perm.size();
            perm.resize((size_t)(base_pos + cnt[NBINS]));
            std::vector<int64_t> at(cnt.begin(), cnt.end() - 1);
            for (int64_t r = s0; r < s1; ++r) {
                if (len[r] > CHUNK) continue;
                perm[(size_t)(base_pos + at[(size_t)bin_of(len[r])]++)] = (int32_t)r;
            }
            // one group per lanes-per-row class: its bins are consecutive, so its rows are
            // sorted by the work of each lane and a warp's 32 / G rows have equal or
            // adjacent lengths (one partial warp per class and segment, not per bin)
            for (int b0 = 0; b0 < NBINS;) {
                const int G = bin_lanes(b0);
                int b1 = b0;
                while (b1 < NBINS && bin_lanes(b1) == G) ++b1;
                const int64_t nrows = cnt[(size_t)b1] - cnt[(size_t)b0];
                if (nrows > 0) {
                    const int64_t nw = ceil_div(nrows, 32 / G);
                    const int64_t gi = (int64_t)groups.size() / 4;
                    if (gi > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "plan: too many bin groups");
                    groups.push_back((int64_t)warp_group.size());
                    groups.push_back(base_pos + cnt[(size_t)b0]);
                    groups.push_back(base_pos + cnt[(size_t)b1]);
                    groups.push_back(G);
                    for (int64_t q = 0; q < nw; ++q) warp_group.push_back((int32_t)gi);
                }
                b0 = b1;
            }
        }
    }
    p->outer_n = outer_n;
    p->nnz = nnz;
    p->max_len = maxlen;
    p->nbin_warps = (int64_t)warp_group.size();
    p->nplanned = binned ? outer_n : (int64_t)hs[0].row.size();
    if (p->nplanned == 0) return GSA_OK;
    size_t bytes = align_up(perm.size() * 4, 256) + align_up(warp_group.size() * 4, 256) +
                   align_up(groups.size() * 8, 256) + align_up(sizeof(gsa_bin_order), 256);
    for (int t = 0; t < 2; ++t)
        bytes += align_up(hs[t].row.size() * 8, 256) + align_up(hs[t].first.size() * 4, 256) +
                 align_up(hs[t].count.size() * 4, 256) + align_up(hs[t].slot.size() * 4, 256) +
                 align_up(mask_nat.size() * 4, 256);
    rc = check_cuda(cudaMalloc(&p->mem, bytes), "plan: device memory");
    if (rc) return rc;
    Carver cv(p->mem);
    auto up = [&](void *dst, const void *src, size_t n, const char *what) {
        if (!rc && n) rc = check_cuda(cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice), what);
    };
    for (int t = 0; t < 2; ++t) {
        gsa_chunk_set &c = t == 0 ? p->nat : p->bin;
        const std::vector<uint32_t> &mask = t == 0 ? mask_nat : mask_bin;
        const HostSet &h2 = hs[t];
        int64_t *d_row = cv.take<int64_t>(h2.row.size());
        int32_t *d_first = cv.take<int32_t>(h2.first.size());
        int32_t *d_count = cv.take<int32_t>(h2.count.size());
        int32_t *d_slot = cv.take<int32_t>(h2.slot.size());
        uint32_t *d_mask = cv.take<uint32_t>(mask.size());
        up(d_row, h2.row.data(), h2.row.size() * 8, "plan: rows");
        up(d_first, h2.first.data(), h2.first.size() * 4, "plan: first");
        up(d_count, h2.count.data(), h2.count.size() * 4, "plan: count");
        up(d_slot, h2.slot.data(), h2.slot.size() * 4, "plan: chunks");
        up(d_mask, mask.data(), mask.size() * 4, "plan: mask");
        c.nlong = (int64_t)h2.row.size();
        c.nchunks = (int64_t)h2.slot.size();
        c.row = d_row;
        c.first = d_first;
        c.count = d_count;
        c.chunk_slot = d_slot;
        c.skip_mask = d_mask;
    }
    int32_t *d_perm = cv.take<int32_t>(perm.size());
    int32_t *d_wg = cv.take<int32_t>(warp_group.size());
    int64_t *d_groups = cv.take<int64_t>(groups.size());
    up(d_perm, perm.data(), perm.size() * 4, "plan: order");
    up(d_wg, warp_group.data(), warp_group.size() * 4, "plan: warp groups");
    up(d_groups, groups.data(), groups.size() * 8, "plan: groups");
    gsa_bin_order *d_view = cv.take<gsa_bin_order>(1);
    if (binned) {
        p->order = gsa_bin_order{p->nbin_warps, d_perm, d_wg, d_groups};
        up(d_view, &p->order, sizeof(gsa_bin_order), "plan: bin view");
    }
    if (rc) return rc;
    if (binned) p->bin_view = d_view;
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
