// Scatter products and the beta pass.
//
// * Compressed scatter: C[idx_j, c] += a_j * (op(B)(o, c) * alpha) for every
//   stored entry j of outer o -- kernel_spmatmul_csr_T!
//   (src/matrix_csr/matrix_csr_kernels.jl:24-45) and kernel_spmatmul_csc_N!
//   (src/matrix_csc/matrix_csc_kernels.jl:1-22).  Those give one work item per
//   outer entry, so one long column serialises a thread.  The default here is the
//   outer-block form of the row-block gather: a warp owns 32 outer entries and gives
//   each G lanes (G from their average length), a lane reads op(B)(o, c) * alpha once
//   per outer entry and adds its entries' products with atomics; with a plan, long
//   outer entries go to warps of their own, chunk by chunk.  ALGO_MERGE cuts the
//   entries into nnz-balanced merge-path tiles instead; a tile first labels each of
//   its entries with its outer index (shared memory), then streams them coalesced.
// * COO: kernel_spmatmul_coo_N! / _T! (src/matrix_coo/matrix_coo_kernels.jl:1-43),
//   one atomic per entry there.  Here each warp takes 32 consecutive entries,
//   reduces runs of equal output rows with a segmented shuffle scan and issues
//   one atomic per run (row-sorted COO: about one per row; any order: correct).
// * rmul_or_fill: LinearAlgebra._rmul_or_fill!(C, beta) as the reference calls
//   it before its atomic kernels (src/matrix_csr/matrix_csr.jl:192).
//
// Complex values use one atomic per component (the reference's KA @atomic
// cannot do Complex, so its CSR-T / CSC-N / COO products skip Complex).
#include "gsa_rows.cuh"

namespace gsa {

template <typename V>
__global__ void rmul_or_fill_kernel(DenseOut<V> C, int64_t rows, int64_t k) {
    int64_t total = rows * k;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t % rows, c = t / rows;
        V *q = C.p + r + c * C.ld;
        if (C.beta_mode == 0) *q = VT<V>::zero();
        else *q = mul(*q, C.beta);
    }
}

template <typename V>
int launch_rmul_or_fill(cudaStream_t s, DenseOut<V> C, int64_t rows, int64_t k) {
    if (C.beta_mode == 1 || rows == 0 || k == 0) return GSA_OK;
    if (C.beta_mode == 0 && (k == 1 || C.ld == rows))  // fill!(C, 0) of one contiguous range:
        return check_cuda(cudaMemsetAsync(C.p, 0, (size_t)rows * (size_t)k * sizeof(V), s),  // +0 bytes
                          "zero fill");
    int64_t blocks = ceil_div(rows * k, 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    rmul_or_fill_kernel<V><<<(unsigned)blocks, 256, 0, s>>>(C, rows, k);
    return check_cuda(cudaGetLastError(), "rmul_or_fill_kernel");
}

// ---------------------------------------------------------------------------
template <typename V> struct ScatterShape {
    static constexpr int THREADS = 256;
    static constexpr int IPT = 8;
    static constexpr int TILE = THREADS * IPT;
};

template <typename V, typename I>
__global__ void __launch_bounds__(ScatterShape<V>::THREADS)
scatter_merge_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C,
                     const int64_t *__restrict__ coords) {
    constexpr int THREADS = ScatterShape<V>::THREADS;
    constexpr int IPT = ScatterShape<V>::IPT;
    constexpr int TILE = ScatterShape<V>::TILE;
    __shared__ int s_rowend[TILE];
    __shared__ int s_outer[TILE];

    const int64_t tile = blockIdx.x;
    const int64_t total = a.outer_n + a.nnz;
    const int64_t d0 = tile * TILE;
    const int64_t d1 = d0 + TILE < total ? d0 + TILE : total;
    const int64_t rs = coords[tile], re = coords[tile + 1];
    const int64_t js = d0 - rs, je = d1 - re;
    const int64_t tile_rows64 = re - rs, tile_nnz64 = je - js;
    if (tile_rows64 < 0 || tile_nnz64 < 0 || tile_rows64 + tile_nnz64 > TILE) return;
    const int tile_rows = (int)tile_rows64, tile_nnz = (int)tile_nnz64;
    const int tid = threadIdx.x;

    for (int e = tid; e < tile_rows; e += THREADS)
        s_rowend[e] = (int)((int64_t)__ldg(a.ptr + rs + 1 + e) - a.base - js);
    __syncthreads();

    // label every entry of the tile with its (local) outer index
    const int items = tile_rows + tile_nnz;
    int d = tid * IPT < items ? tid * IPT : items;
    int lo = d - tile_nnz > 0 ? d - tile_nnz : 0;
    int hi = d < tile_rows ? d : tile_rows;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s_rowend[mid] + mid < d) lo = mid + 1;
        else hi = mid;
    }
    int i = lo, j = d - lo;
#pragma unroll
    for (int step = 0; step < IPT; ++step) {
        if (i < tile_rows && s_rowend[i] <= j) ++i;
        else if (j < tile_nnz) s_outer[j++] = i;
    }
    __syncthreads();

    I idx[IPT];
    V av[IPT];
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        int e = tid + u * THREADS;
        if (e < tile_nnz) {
            idx[u] = ld_stream(a.idx + js + e);
            av[u] = conj_if(ld_stream(a.val + js + e), a.conjA);
        }
    }
    for (int64_t c = 0; c < k; ++c) {
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            int e = tid + u * THREADS;
            int64_t r = (int64_t)idx[u] - a.base;
            if (e < tile_nnz && (uint64_t)r < (uint64_t)a.inner_n) {
                V axj = mul(B.at(rs + s_outer[e], c), C.alpha);
                atomic_add(C.p + r + c * C.ld, mul(av[u], axj));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Outer-block scatter (the default).

// op(B)(o, c) * alpha, without the multiply when alpha == 1 of a real type (exact).
template <typename V>
__device__ __forceinline__ V alpha_times(const DenseOut<V> &C, V b) {
    return C.alpha_one ? b : mul(b, C.alpha);
}

// C[idx_j, c0 + c] += conj?(a_j) * xa[c] for j = jb, jb+S, ... < je; entries whose index
// falls outside C's rows are skipped.  U entries are loaded before their atomics are
// issued, so a lane keeps U loads in flight instead of one load per atomic.
template <typename V, typename I, int KC, int S, int U>
__device__ __forceinline__ void scatter_range(const CompressedArgs<V, I> &a, const DenseOut<V> &C,
                                              Off<I> j, Off<I> je, int64_t c0, int64_t k,
                                              const V (&xa)[KC]) {
    using O = Off<I>;
    const I *__restrict__ idx = a.idx;
    const V *__restrict__ val = a.val;
    V *__restrict__ out = C.p;
    const O inner = sizeof(O) == 8 ? (O)a.inner_n
                                   : (O)(a.inner_n < 0xffffffffLL ? a.inner_n : 0xffffffffLL);
    const O base = (O)a.base;
    if (U > 1) {
        for (; j + (O)((U - 1) * S) < je; j += U * S) {
            O r[U];
            V av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                r[u] = (O)ld_stream(idx + j + u * S) - base;
                av[u] = conj_if(ld_stream(val + j + u * S), a.conjA);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (r[u] >= inner) continue;
#pragma unroll
                for (int c = 0; c < KC; ++c)
                    if (KC == 1 || c0 + c < k) atomic_add(out + (int64_t)r[u] + (c0 + c) * C.ld, mul(av[u], xa[c]));
            }
        }
    }
    for (; j < je; j += S) {
        const O r = (O)ld_stream(idx + j) - base;
        const V av = conj_if(ld_stream(val + j), a.conjA);
        if (r >= inner) continue;
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (KC == 1 || c0 + c < k) atomic_add(out + (int64_t)r + (c0 + c) * C.ld, mul(av, xa[c]));
    }
}

// The 32 outer entries of one warp, G lanes each (as warp_rows, scattering).
template <typename V, typename I, int KC, int G>
__device__ __forceinline__ void scatter_rows(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                             const DenseOut<V> &C, int64_t c0, int64_t row0, Off<I> b,
                                             Off<I> e) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    constexpr int RPP = 32 / G;
#pragma unroll 1
    for (int p = 0; p < G; ++p) {
        const int q = p * RPP + lane / G;
        const O qb = G == 1 ? b : (O)__shfl_sync(0xffffffffu, b, q);
        const O qe = G == 1 ? e : (O)__shfl_sync(0xffffffffu, e, q);
        if (qb >= qe) continue;  // empty, planned, or past the last outer entry
        const int64_t o = row0 + q;
        V xa[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c)
            xa[c] = (KC == 1 || c0 + c < k) ? alpha_times(C, B.at(o, c0 + c)) : VT<V>::zero();
        scatter_range<V, I, KC, G, (G == 1 ? 4 : 2)>(a, C, qb + (O)(lane % G), qe, c0, k, xa);
    }
}

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS)
scatter_block_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t ncg,
                     int64_t nrb, PlanRows P) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const unsigned cta = blockIdx.x;
    const unsigned cg = ncg == 1 ? 0u : cta % (unsigned)ncg;
    const int64_t unit = ncg == 1 ? (int64_t)cta : (int64_t)(cta / (unsigned)ncg);
    const int64_t c0 = (int64_t)cg * KC;
    if (unit >= nrb) {
        // planned outer entries: a warp per chunk, straight to the atomics
        const int64_t chunk = (unit - nrb) * RB_WARPS + (threadIdx.x >> 5);
        if (chunk >= P.nchunks) return;
        const int slot = P.chunk_slot[chunk];
        const int64_t o = P.row[slot];
        const O nz = (O)a.nnz, base = (O)a.base;
        O rb = (O)__ldg(a.ptr + o) - base;
        O re = (O)__ldg(a.ptr + o + 1) - base;
        rb = rb < nz ? rb : nz;
        re = re < nz ? re : nz;
        const O jb = rb + (O)(chunk - P.first[slot]) * (O)CHUNK;
        const O je = jb < re && re - jb > (O)CHUNK ? jb + (O)CHUNK : re;
        if (jb >= je) return;
        V xa[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c)
            xa[c] = (KC == 1 || c0 + c < k) ? alpha_times(C, B.at(o, c0 + c)) : VT<V>::zero();
        scatter_range<V, I, KC, 32, UNROLL>(a, C, jb + (O)lane, je, c0, k, xa);
        return;
    }
    const int64_t row0 = unit * RB_THREADS + (threadIdx.x & ~31);
    Off<I> b, e;
    int skip;
    const int64_t avg = warp_extent(a, row0, P.skip_mask, b, e, skip);
    dispatch_lanes(avg, G1_AVG, [&](auto g) {
        scatter_rows<V, I, KC, decltype(g)::value>(a, k, B, C, c0, row0, b, e);
    });
}

// ---------------------------------------------------------------------------
// Window scatter (GSA_ALGO_VECTOR, one right-hand side): a thread per outer entry, and the
// products whose output row lies within WIN_HALO rows of the CTA's own outer range -- the
// band of a banded matrix, where the outer entries of one CTA hit the same rows -- summed in
// a shared-memory window first, then added with one atomic per touched row of the window.
// Products outside the window go to the global atomics directly.  The partial sums of the
// window are combined in shared memory: the adds move from the L2 atomic units to the SM.
constexpr int WIN_THREADS = 128;
constexpr int WIN_HALO = 64;
constexpr int WIN_ROWS = WIN_THREADS + 2 * WIN_HALO;

__device__ __forceinline__ void smem_add(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void smem_add(double *p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void smem_add(cf32 *p, cf32 v) { atomicAdd(&p->re, v.re); atomicAdd(&p->im, v.im); }
__device__ __forceinline__ void smem_add(cf64 *p, cf64 v) { atomicAdd(&p->re, v.re); atomicAdd(&p->im, v.im); }
__device__ __forceinline__ void smem_add(int32_t *p, int32_t v) { atomicAdd((int *)p, (int)v); }
__device__ __forceinline__ void smem_add(int64_t *p, int64_t v) {
    atomicAdd((unsigned long long *)p, (unsigned long long)v);
}

template <typename V, typename I>
__global__ void __launch_bounds__(WIN_THREADS)
scatter_window_kernel(CompressedArgs<V, I> a, DenseIn<V> B, DenseOut<V> C, int64_t out_rows) {
    using O = Off<I>;
    __shared__ V s_acc[WIN_ROWS];
    __shared__ uint32_t s_touched[WIN_ROWS / 32];
    const int tid = threadIdx.x;
    const int64_t o0 = (int64_t)blockIdx.x * WIN_THREADS;
    const int64_t lo = o0 - WIN_HALO;  // output row of window slot 0 (may be negative)
    for (int w = tid; w < WIN_ROWS; w += WIN_THREADS) s_acc[w] = VT<V>::zero();
    if (tid < WIN_ROWS / 32) s_touched[tid] = 0u;
    __syncthreads();
    const int64_t o = o0 + tid;
    if (o < a.outer_n) {
        const O nz = (O)a.nnz, base = (O)a.base;
        O j = (O)__ldg(a.ptr + o) - base;
        O je = (O)__ldg(a.ptr + o + 1) - base;
        j = j < nz ? j : nz;
        je = je < nz ? je : nz;
        const V xa = alpha_times(C, B.at(o, 0));
        const uint64_t rows = (uint64_t)out_rows;
        for (; j < je; ++j) {
            const int64_t r = (int64_t)ld_stream(a.idx + j) - a.base;
            const V pr = mul(conj_if(ld_stream(a.val + j), a.conjA), xa);
            if ((uint64_t)r >= rows) continue;
            const int64_t w = r - lo;
            if (w >= 0 && w < WIN_ROWS) {
                smem_add(&s_acc[w], pr);
                atomicOr(&s_touched[w >> 5], 1u << (w & 31));
            } else {
                atomic_add(C.p + r, pr);
            }
        }
    }
    __syncthreads();
    for (int w = tid; w < WIN_ROWS; w += WIN_THREADS)
        if ((s_touched[w >> 5] >> (w & 31)) & 1u) atomic_add(C.p + (lo + w), s_acc[w]);
}

template <typename V, typename I>
int launch_scatter_block(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                         DenseOut<V> C, const Plan *plan) {
    const int64_t nrb = ceil_div(a.outer_n, RB_THREADS);
    int KC = get_spmm_columns();
    if (KC == 0) KC = sizeof(V) >= 16 ? 2 : 4;
    if (k == 1) KC = 1;
    if (KC > k) KC = k <= 2 ? 2 : (k <= 4 ? 4 : 8);
    const int64_t ncg = ceil_div(k, KC);
    PlanRows P{};
    int64_t units = nrb;
    if (plan && plan->nat.nlong > 0) {  // natural order: the natural chunk set
        if (plan->outer_n != a.outer_n || plan->nnz != a.nnz)
            return fail(GSA_ERR_INVALID_ARG, "plan was made for another structure");
        P = plan_rows(plan->nat);
        units += ceil_div(plan->nat.nchunks, RB_WARPS);
    }
    const int64_t blocks = units * ncg;
    if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many outer entries");
    timer_before(s);
    if (KC == 1) scatter_block_kernel<V, I, 1><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, P);
    else if (KC == 2) scatter_block_kernel<V, I, 2><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, P);
    else if (KC == 4) scatter_block_kernel<V, I, 4><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, P);
    else scatter_block_kernel<V, I, 8><<<(unsigned)blocks, RB_THREADS, 0, s>>>(a, k, B, C, ncg, nrb, P);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "scatter_block_kernel");
}

template <typename V, typename I>
size_t scatter_workspace_size(int64_t outer_n, int64_t nnz, int64_t k, int algo) {
    if (algo != GSA_ALGO_MERGE) return 0;
    if (outer_n == 0 || nnz == 0 || k == 0) return 0;
    int64_t T = ceil_div(outer_n + nnz, ScatterShape<V>::TILE);
    return align_up((size_t)(T + 1) * sizeof(int64_t), 256);
}

template <typename V, typename I>
int launch_scatter(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                   DenseOut<V> C, int64_t out_rows, int algo, const Plan *plan, void *ws,
                   size_t ws_bytes) {
    int rc = launch_rmul_or_fill<V>(s, C, out_rows, k);
    if (rc) return rc;
    if (a.outer_n == 0 || a.nnz == 0 || k == 0) return GSA_OK;
    if (algo == GSA_ALGO_VECTOR && k == 1) {
        const int64_t blocks = ceil_div(a.outer_n, WIN_THREADS);
        if (blocks > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many outer entries");
        timer_before(s);
        scatter_window_kernel<V, I><<<(unsigned)blocks, WIN_THREADS, 0, s>>>(a, B, C, out_rows);
        timer_after(s);
        return check_cuda(cudaGetLastError(), "scatter_window_kernel");
    }
    if (algo != GSA_ALGO_MERGE) return launch_scatter_block<V, I>(s, a, k, B, C, plan);
    constexpr int TILE = ScatterShape<V>::TILE;
    const int64_t T = ceil_div(a.outer_n + a.nnz, TILE);
    if (ws_bytes < scatter_workspace_size<V, I>(a.outer_n, a.nnz, k, algo))
        return fail(GSA_ERR_INVALID_ARG, "scatter workspace too small");
    if (T > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many tiles");
    int64_t *coords = (int64_t *)ws;
    rc = launch_merge_partition<I>(s, a.ptr, a.base, a.outer_n, a.nnz, TILE, T, coords);
    if (rc) return rc;
    timer_before(s);
    scatter_merge_kernel<V, I><<<(unsigned)T, ScatterShape<V>::THREADS, 0, s>>>(a, k, B, C, coords);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "scatter_merge_kernel");
}

// ---------------------------------------------------------------------------
// COO: each warp takes 32 consecutive entries at a time; a segmented scan over runs of
// equal adjacent output indices leaves each run's sum in its last lane, which adds it
// with one atomic.  Equal indices that are not adjacent form separate runs.
// Six resident CTAs of 256 threads (40 registers, no spills for any value type): the power-law
// ComplexF64 COO in random order 293 us against 309 us unbounded (48 registers) on one GB300, and
// 375 us with 8 (32 registers, spilling).
#ifndef GSA_COO_MIN_BLOCKS
#define GSA_COO_MIN_BLOCKS 6
#endif
template <typename V, typename I>
__global__ void __launch_bounds__(256, GSA_COO_MIN_BLOCKS)
coo_kernel(int64_t nnz, const I *__restrict__ out_idx, const I *__restrict__ in_idx,
           const V *__restrict__ val, int base, bool conjA, int64_t k, DenseIn<V> B,
           DenseOut<V> C, int64_t out_rows, int64_t in_rows) {
    // op(B)(in, c) * alpha (alpha == 1 of a real type needs no multiply: exact)
    auto xa = [&](int64_t in, int64_t c) -> V {
        const V x = B.at(in, c);
        return C.alpha_one ? x : mul(x, C.alpha);
    };
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t g = warp; g * 32 < nnz; g += nwarps) {
        const int64_t e = g * 32 + lane;
        bool valid = e < nnz;
        int64_t key = -1, in = 0;
        V av = VT<V>::zero();
        if (valid) {
            key = (int64_t)ld_stream(out_idx + e) - base;
            in = (int64_t)ld_stream(in_idx + e) - base;
            av = conj_if(ld_stream(val + e), conjA);
            // entries outside the matrix are skipped, never read or written
            if ((uint64_t)key >= (uint64_t)out_rows || (uint64_t)in >= (uint64_t)in_rows) {
                valid = false;
                key = -1;
            }
        }
        // runs of equal adjacent keys: a run starts where the previous lane's key differs
        const int64_t prev_key = __shfl_up_sync(0xffffffffu, key, 1);
        const int64_t next_key = __shfl_down_sync(0xffffffffu, key, 1);
        const bool tail = valid && (lane == 31 || next_key != key);
        // no run longer than one entry in this warp (COO in random order): every valid entry
        // is its own tail, and the segmented sum -- five rounds of adds on the FP64 pipe -- is
        // skipped (warp-uniform)
        const bool runs = __any_sync(0xffffffffu, valid && !tail);
        if (!runs) {
            for (int64_t c = 0; c < k; ++c)
                if (valid) atomic_add(C.p + key + c * C.ld, mul(av, xa(in, c)));
            continue;
        }
        int run_start = (lane == 0 || prev_key != key) ? lane : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int o = __shfl_up_sync(0xffffffffu, run_start, off);
            if (lane >= off && o > run_start) run_start = o;
        }
        for (int64_t c = 0; c < k; ++c) {
            V v = valid ? mul(av, xa(in, c)) : VT<V>::zero();
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                V ov = shfl_up(v, off);
                if (lane - off >= run_start) v = add(ov, v);
            }
            if (tail) atomic_add(C.p + key + c * C.ld, v);
        }
    }
}

template <typename V, typename I>
int launch_coo(cudaStream_t s, int64_t nnz, const I *out_idx, const I *in_idx, const V *val,
               int base, bool conjA, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t out_rows,
               int64_t in_rows) {
    int rc = launch_rmul_or_fill<V>(s, C, out_rows, k);
    if (rc) return rc;
    if (nnz == 0 || k == 0) return GSA_OK;
    int64_t warps = ceil_div(nnz, 32);
    int64_t blocks = ceil_div(warps, 8);
    if (blocks > 152 * 16) blocks = 152 * 16;
    timer_before(s);
    coo_kernel<V, I><<<(unsigned)blocks, 256, 0, s>>>(nnz, out_idx, in_idx, val, base, conjA, k, B,
                                                       C, out_rows, in_rows);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "coo_kernel");
}

#define GSA_INST_SCATTER(V, I)                                                                  \
    template int launch_scatter<V, I>(cudaStream_t, const CompressedArgs<V, I> &, int64_t,      \
                                      DenseIn<V>, DenseOut<V>, int64_t, int, const Plan *,      \
                                      void *, size_t);                                          \
    template size_t scatter_workspace_size<V, I>(int64_t, int64_t, int64_t, int);               \
    template int launch_coo<V, I>(cudaStream_t, int64_t, const I *, const I *, const V *, int, \
                                  bool, int64_t, DenseIn<V>, DenseOut<V>, int64_t, int64_t);
GSA_INST_SCATTER(float, int32_t)
GSA_INST_SCATTER(float, int64_t)
GSA_INST_SCATTER(double, int32_t)
GSA_INST_SCATTER(double, int64_t)
GSA_INST_SCATTER(cf32, int32_t)
GSA_INST_SCATTER(cf32, int64_t)
GSA_INST_SCATTER(cf64, int32_t)
GSA_INST_SCATTER(cf64, int64_t)
GSA_INST_SCATTER(int32_t, int32_t)
GSA_INST_SCATTER(int32_t, int64_t)
GSA_INST_SCATTER(int64_t, int32_t)
GSA_INST_SCATTER(int64_t, int64_t)

template int launch_rmul_or_fill<float>(cudaStream_t, DenseOut<float>, int64_t, int64_t);
template int launch_rmul_or_fill<double>(cudaStream_t, DenseOut<double>, int64_t, int64_t);
template int launch_rmul_or_fill<cf32>(cudaStream_t, DenseOut<cf32>, int64_t, int64_t);
template int launch_rmul_or_fill<cf64>(cudaStream_t, DenseOut<cf64>, int64_t, int64_t);
template int launch_rmul_or_fill<int32_t>(cudaStream_t, DenseOut<int32_t>, int64_t, int64_t);
template int launch_rmul_or_fill<int64_t>(cudaStream_t, DenseOut<int64_t>, int64_t, int64_t);

}  // namespace gsa
