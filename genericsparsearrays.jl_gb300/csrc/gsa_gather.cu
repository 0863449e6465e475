// Row-gather products: C[o, c] = beta*C[o, c] + alpha * sum_j a_j * op(B)(idx_j, c)
// over the compressed outer dimension.  This is the work of
// kernel_spmatmul_csr_N! (src/matrix_csr/matrix_csr_kernels.jl:1-22) and
// kernel_spmatmul_csc_T! (src/matrix_csc/matrix_csc_kernels.jl:24-45), which
// give one work item per (row, rhs column) and walk the row serially.
//
// Here the work is split instead into equal tiles of the merge path of the
// outer end offsets and the stored entries (Merrill & Garland, "Merge-based
// parallel sparse matrix-vector multiplication", SC'16): every CTA consumes
// THREADS*IPT items (an item is one stored entry or one row end), so a
// 50,000-entry row costs the same per CTA as 5,000 ten-entry rows.
//
//   1. merge_partition_kernel: tile boundary coordinates (one binary search each)
//   2. gather_merge_kernel: per tile, stage products a_j * B(idx_j, c) in shared
//      memory with coalesced streaming loads, run the per-thread merge walk,
//      combine per-thread partial rows with a segmented scan, write completed
//      rows coalesced (beta/alpha fused) and publish the partial of the row
//      that is still open at the tile's end
//   3. gather_fixup_kernel: add the open-row partials to their rows, in tile
//      order (deterministic; no atomics anywhere on this path)
//
// A second kernel, gather_vector_kernel, gives each row a group of G lanes;
// it needs no workspace and suits short rows of even length.
#include "gsa_internal.cuh"

namespace gsa {

// ---------------------------------------------------------------------------
// Merge-path partition.  f(r) = end(r) + r is strictly increasing; the tile
// boundary on diagonal d consumes the outer entries r with f(r) < d.
template <typename I>
__global__ void merge_partition_kernel(const I *__restrict__ ptr, int base, int64_t outer_n,
                                       int64_t nnz, int64_t tile_items, int64_t num_tiles,
                                       int64_t *__restrict__ coords) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > num_tiles) return;
    int64_t total = outer_n + nnz;
    int64_t d = t * tile_items;
    if (d > total) d = total;
    int64_t lo = d - nnz > 0 ? d - nnz : 0;
    int64_t hi = d < outer_n ? d : outer_n;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        int64_t f = (int64_t)__ldg(ptr + mid + 1) - base + mid;
        if (f < d) lo = mid + 1;
        else hi = mid;
    }
    coords[t] = lo;
}

template <typename I>
int launch_merge_partition(cudaStream_t s, const I *ptr, int base, int64_t outer_n, int64_t nnz,
                           int64_t tile_items, int64_t num_tiles, int64_t *coords) {
    int threads = 256;
    int64_t blocks = ceil_div(num_tiles + 1, threads);
    merge_partition_kernel<I><<<(unsigned)blocks, threads, 0, s>>>(ptr, base, outer_n, nnz,
                                                                  tile_items, num_tiles, coords);
    return check_cuda(cudaGetLastError(), "merge_partition_kernel");
}
template int launch_merge_partition<int32_t>(cudaStream_t, const int32_t *, int, int64_t, int64_t,
                                             int64_t, int64_t, int64_t *);
template int launch_merge_partition<int64_t>(cudaStream_t, const int64_t *, int, int64_t, int64_t,
                                             int64_t, int64_t, int64_t *);

// ---------------------------------------------------------------------------
// Tile shape per value size: 256 threads; items per thread chosen so the
// staged products fit comfortably in shared memory with several CTAs per SM.
template <typename V> struct GatherShape {
    static constexpr int THREADS = 256;
    static constexpr int IPT = sizeof(V) >= 16 ? 5 : 8;
    static constexpr int TILE = THREADS * IPT;
};

// Block-wide inclusive segmented scan of (key, v) over threads in thread order;
// keys are non-decreasing across threads.  Returns this thread's inclusive sum
// over the run of equal keys that ends at it.
template <typename V, int THREADS>
__device__ __forceinline__ V block_segscan(int key, V v, int *s_wfirst, int *s_wlast, V *s_wtot,
                                           V *s_wpre) {
    constexpr int WARPS = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        V ov = shfl_up(v, off);
        int ok = __shfl_up_sync(0xffffffffu, key, off);
        if (lane >= off && ok == key) v = add(ov, v);
    }
    if (lane == 31) { s_wlast[warp] = key; s_wtot[warp] = v; }
    if (lane == 0) s_wfirst[warp] = key;
    __syncthreads();
    if (threadIdx.x < WARPS) {
        int w = threadIdx.x, K = s_wfirst[w];
        V p = VT<V>::zero();
        for (int w2 = w - 1; w2 >= 0; --w2) {
            if (s_wlast[w2] != K) break;
            p = add(s_wtot[w2], p);
            if (s_wfirst[w2] != K) break;
        }
        s_wpre[w] = p;
    }
    __syncthreads();
    if (key == s_wfirst[warp]) v = add(s_wpre[warp], v);
    return v;
}

// MULTI: k > 1 right-hand sides; the tile's indices and values are staged in
// (dynamic) shared memory once and reused for every column.
template <typename V, typename I, bool MULTI>
__global__ void __launch_bounds__(GatherShape<V>::THREADS)
gather_merge_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C,
                    const int64_t *__restrict__ coords, int64_t *__restrict__ carry_row,
                    V *__restrict__ carry_val) {
    constexpr int THREADS = GatherShape<V>::THREADS;
    constexpr int IPT = GatherShape<V>::IPT;
    constexpr int TILE = GatherShape<V>::TILE;
    constexpr int WARPS = THREADS / 32;
    __shared__ int s_rowend[TILE];
    __shared__ V s_val[TILE];  // products in [0, tile_nnz), row sums in [tile_nnz, +tile_rows)
    __shared__ V s_scan[THREADS];
    __shared__ int s_wfirst[WARPS], s_wlast[WARPS];
    __shared__ V s_wtot[WARPS], s_wpre[WARPS];
    extern __shared__ __align__(16) unsigned char s_dyn[];

    const int64_t tile = blockIdx.x;
    const int64_t total = a.outer_n + a.nnz;
    const int64_t d0 = tile * TILE;
    const int64_t d1 = d0 + TILE < total ? d0 + TILE : total;
    const int64_t rs = coords[tile], re = coords[tile + 1];
    const int64_t js = d0 - rs, je = d1 - re;
    const int64_t tile_rows64 = re - rs, tile_nnz64 = je - js;
    // A malformed pointer array can only make a tile wrong, never out of bounds.
    if (tile_rows64 < 0 || tile_nnz64 < 0 || tile_rows64 + tile_nnz64 > TILE) {
        if (threadIdx.x == 0) carry_row[tile] = -1;
        return;
    }
    const int tile_rows = (int)tile_rows64, tile_nnz = (int)tile_nnz64;
    const int tid = threadIdx.x;

    for (int e = tid; e < tile_rows; e += THREADS)
        s_rowend[e] = (int)((int64_t)__ldg(a.ptr + rs + 1 + e) - a.base - js);

    V *s_a = reinterpret_cast<V *>(s_dyn);
    I *s_col = reinterpret_cast<I *>(s_dyn + sizeof(V) * TILE);
    if (MULTI) {
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            int e = tid + u * THREADS;
            if (e < tile_nnz) {
                s_col[e] = ld_stream(a.idx + js + e);
                s_a[e] = conj_if(ld_stream(a.val + js + e), a.conjA);
            }
        }
        __syncthreads();
    }

    for (int64_t c = 0; c < k; ++c) {
        // 1. products, staged in shared memory
        if (MULTI) {
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                int e = tid + u * THREADS;
                if (e < tile_nnz) {
                    int64_t ci = (int64_t)s_col[e] - a.base;
                    s_val[e] = (uint64_t)ci < (uint64_t)a.inner_n ? mul(s_a[e], B.at(ci, c))
                                                                   : VT<V>::zero();
                }
            }
        } else {
            I col[IPT];
            V av[IPT];
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                int e = tid + u * THREADS;
                if (e < tile_nnz) {
                    col[u] = ld_stream(a.idx + js + e);
                    av[u] = ld_stream(a.val + js + e);
                }
            }
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                int e = tid + u * THREADS;
                if (e < tile_nnz) {
                    int64_t ci = (int64_t)col[u] - a.base;
                    s_val[e] = (uint64_t)ci < (uint64_t)a.inner_n
                                   ? mul(conj_if(av[u], a.conjA), B.at(ci, c))
                                   : VT<V>::zero();
                }
            }
        }
        __syncthreads();

        // 2. this thread's IPT items of the tile's merge path
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
        const int i_start = i;
        V acc = VT<V>::zero();
#pragma unroll
        for (int step = 0; step < IPT; ++step) {
            if (i < tile_rows && s_rowend[i] <= j) {
                s_val[tile_nnz + i] = acc;
                acc = VT<V>::zero();
                ++i;
            } else if (j < tile_nnz) {
                acc = add(acc, s_val[j]);
                ++j;
            }
        }

        // 3. partial rows that cross thread boundaries
        V incl = block_segscan<V, THREADS>(i, acc, s_wfirst, s_wlast, s_wtot, s_wpre);
        s_scan[tid] = incl;
        __syncthreads();
        if (tid > 0 && i > i_start)
            s_val[tile_nnz + i_start] = add(s_scan[tid - 1], s_val[tile_nnz + i_start]);
        __syncthreads();

        // 4. completed rows, coalesced, with beta/alpha fused
        for (int e = tid; e < tile_rows; e += THREADS) C.store(rs + e, c, s_val[tile_nnz + e]);

        // 5. the open row's partial for the fixup pass
        if (tid == THREADS - 1) {
            int open_start = tile_rows > 0 ? s_rowend[tile_rows - 1] : 0;
            bool has = (re < a.outer_n) && (tile_nnz > open_start);
            if (c == 0) carry_row[tile] = has ? re : -1;
            carry_val[tile * k + c] = incl;
        }
        __syncthreads();
    }
}

// Adds every open-row partial to its row, summing runs of tiles that carry the
// same row in tile order.  Runs after gather_merge_kernel on the same stream.
template <typename V>
__global__ void gather_fixup_kernel(int64_t num_tiles, int64_t k,
                                    const int64_t *__restrict__ carry_row,
                                    const V *__restrict__ carry_val, DenseOut<V> C) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= num_tiles) return;
    int64_t r = carry_row[t];
    if (r < 0) return;
    if (t > 0 && carry_row[t - 1] == r) return;
    for (int64_t c = 0; c < k; ++c) {
        V sum = carry_val[t * k + c];
        for (int64_t t2 = t + 1; t2 < num_tiles && carry_row[t2] == r; ++t2)
            sum = add(sum, carry_val[t2 * k + c]);
        C.accumulate(r, c, mul(sum, C.alpha));
    }
}

// ---------------------------------------------------------------------------
// A group of G lanes per row; lanes stride the row and reduce with shuffles.
template <typename V, typename I, int G>
__global__ void __launch_bounds__(256)
gather_vector_kernel(CompressedArgs<V, I> a, int64_t k, DenseIn<V> B, DenseOut<V> C) {
    const int lane = threadIdx.x % G;
    const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
    for (int64_t row = (int64_t)blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
         row < a.outer_n; row += groups) {
        int64_t start = (int64_t)__ldg(a.ptr + row) - a.base;
        int64_t end = (int64_t)__ldg(a.ptr + row + 1) - a.base;
        start = start < 0 ? 0 : start;
        end = end > a.nnz ? a.nnz : end;
        for (int64_t c = 0; c < k; ++c) {
            V acc = VT<V>::zero();
            for (int64_t j = start + lane; j < end; j += G) {
                int64_t ci = (int64_t)ld_stream(a.idx + j) - a.base;
                if ((uint64_t)ci < (uint64_t)a.inner_n)
                    acc = mac(acc, conj_if(ld_stream(a.val + j), a.conjA), B.at(ci, c));
            }
#pragma unroll
            for (int m = G / 2; m > 0; m >>= 1) acc = add(acc, shfl_xor(acc, m, G));
            if (lane == 0) C.store(row, c, acc);
        }
    }
}

// ---------------------------------------------------------------------------
template <typename V, typename I>
static int64_t gather_num_tiles(int64_t outer_n, int64_t nnz) {
    return ceil_div(outer_n + nnz, GatherShape<V>::TILE);
}

template <typename V, typename I>
size_t gather_workspace_size(int64_t outer_n, int64_t nnz, int64_t k, int algo, const Plan *plan) {
    if (algo == GSA_ALGO_AUTO) return rowblock_workspace_size(plan, sizeof(V), k);
    if (algo == GSA_ALGO_VECTOR || outer_n == 0 || k == 0) return 0;
    if (algo == GSA_ALGO_PIPE) return k == 1 ? spmv_pipe_workspace_size<V, I>(outer_n, nnz) : 0;
    int64_t T = gather_num_tiles<V, I>(outer_n, nnz);
    Carver cv(nullptr);
    cv.take<int64_t>(T + 1);
    cv.take<int64_t>(T);
    cv.take<V>((size_t)(T * k));
    return align_up(cv.off, 256);
}

template <typename V, typename I, int G>
static int launch_vector_g(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k,
                           DenseIn<V> B, DenseOut<V> C) {
    int threads = 256;
    int64_t groups_per_block = threads / G;
    int64_t blocks = ceil_div(a.outer_n, groups_per_block);
    int64_t cap = 152 * 64;
    if (blocks > cap) blocks = cap;
    timer_before(s);
    gather_vector_kernel<V, I, G><<<(unsigned)blocks, threads, 0, s>>>(a, k, B, C);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "gather_vector_kernel");
}

template <typename V, typename I>
int launch_gather(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                  DenseOut<V> C, int algo, const Plan *plan, void *ws, size_t ws_bytes) {
    if (a.outer_n == 0 || k == 0) return GSA_OK;
    if (algo == GSA_ALGO_VECTOR) {
        double avg = a.outer_n ? (double)a.nnz / (double)a.outer_n : 0.0;
        if (avg <= 2) return launch_vector_g<V, I, 2>(s, a, k, B, C);
        if (avg <= 4) return launch_vector_g<V, I, 4>(s, a, k, B, C);
        if (avg <= 8) return launch_vector_g<V, I, 8>(s, a, k, B, C);
        if (avg <= 16) return launch_vector_g<V, I, 16>(s, a, k, B, C);
        return launch_vector_g<V, I, 32>(s, a, k, B, C);
    }
    if (algo == GSA_ALGO_AUTO) return launch_rowblock<V, I>(s, a, k, B, C, plan, ws, ws_bytes);
    if (algo == GSA_ALGO_PIPE) {
        if (k != 1) return fail(GSA_ERR_UNSUPPORTED, "GSA_ALGO_PIPE takes one right-hand side");
        return launch_spmv_pipe<V, I>(s, a, B, C, ws, ws_bytes);
    }
    constexpr int TILE = GatherShape<V>::TILE;
    const int64_t T = gather_num_tiles<V, I>(a.outer_n, a.nnz);
    if (ws_bytes < gather_workspace_size<V, I>(a.outer_n, a.nnz, k, algo, nullptr))
        return fail(GSA_ERR_INVALID_ARG, "gather workspace too small");
    Carver cv(ws);
    int64_t *coords = cv.take<int64_t>(T + 1);
    int64_t *carry_row = cv.take<int64_t>(T);
    V *carry_val = cv.take<V>((size_t)(T * k));
    int rc = launch_merge_partition<I>(s, a.ptr, a.base, a.outer_n, a.nnz, TILE, T, coords);
    if (rc) return rc;
    if (T > 0x7fffffffLL) return fail(GSA_ERR_UNSUPPORTED, "too many tiles");
    timer_before(s);
    if (k == 1) {
        gather_merge_kernel<V, I, false><<<(unsigned)T, GatherShape<V>::THREADS, 0, s>>>(
            a, k, B, C, coords, carry_row, carry_val);
    } else {
        size_t dyn = (sizeof(V) + sizeof(I)) * TILE;
        cudaFuncSetAttribute(gather_merge_kernel<V, I, true>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        gather_merge_kernel<V, I, true><<<(unsigned)T, GatherShape<V>::THREADS, dyn, s>>>(
            a, k, B, C, coords, carry_row, carry_val);
    }
    timer_after(s);
    rc = check_cuda(cudaGetLastError(), "gather_merge_kernel");
    if (rc) return rc;
    gather_fixup_kernel<V><<<(unsigned)ceil_div(T, 256), 256, 0, s>>>(T, k, carry_row, carry_val, C);
    return check_cuda(cudaGetLastError(), "gather_fixup_kernel");
}

#define GSA_INST_GATHER(V, I)                                                                   \
    template int launch_gather<V, I>(cudaStream_t, const CompressedArgs<V, I> &, int64_t,       \
                                     DenseIn<V>, DenseOut<V>, int, const Plan *, void *, size_t); \
    template size_t gather_workspace_size<V, I>(int64_t, int64_t, int64_t, int, const Plan *);
GSA_INST_GATHER(float, int32_t)
GSA_INST_GATHER(float, int64_t)
GSA_INST_GATHER(double, int32_t)
GSA_INST_GATHER(double, int64_t)
GSA_INST_GATHER(cf32, int32_t)
GSA_INST_GATHER(cf32, int64_t)
GSA_INST_GATHER(cf64, int32_t)
GSA_INST_GATHER(cf64, int64_t)
GSA_INST_GATHER(int32_t, int32_t)
GSA_INST_GATHER(int32_t, int64_t)
GSA_INST_GATHER(int64_t, int32_t)
GSA_INST_GATHER(int64_t, int64_t)

}  // namespace gsa
