// Grouped products: many CSR SpMV/SpMM products C_i = beta_i C_i + alpha_i A_i B_i in one
// launch.  A plain call launches one kernel per product (the reference's mul! launches
// one KA kernel per call, src/matrix_csr/matrix_csr.jl:194-206); for thousands of small
// matrices of uneven size the launches, not the bytes, set the time.
//
// The work list is implicit: item i owns tiles [first_tile_i, first_tile_i + tiles_i),
// tiles_i = ceil(m_i / 128) row blocks -- or, for an item that carries its plan's bin
// order, ceil(bin_warps_i / 4) CTAs of bin-order warps -- x ceil(k_i / KC) column groups
// (host-side prefix, gsa_grouped_tiles).  A persistent grid (SMs x resident CTAs) walks the tiles; a CTA
// finds its item by binary search over first_tile, then its warps run the same row
// code as the single-product kernel (gsa_rows.cuh: G lanes per row chosen per warp).
// A batch object (gsa_batch_*) keeps the item array on the device and can replay the
// launch from a captured CUDA graph.
#include <new>
#include <vector>

#include "gsa_rows.cuh"

namespace gsa {

static_assert(sizeof(gsa_group_item) == 144, "gsa_group_item layout");

// One value of V from an item's alpha/beta bytes (8-byte loads: the bytes are 8-aligned).
template <typename V>
__device__ __forceinline__ V scalar_at(const unsigned char *p) {
    union { V v; unsigned long long w[sizeof(V) >= 8 ? sizeof(V) / 8 : 1]; unsigned int h; } u;
    if (sizeof(V) >= 8) {
#pragma unroll
        for (int i = 0; i < (int)(sizeof(V) / 8); ++i) u.w[i] = __ldg((const unsigned long long *)p + i);
    } else {
        u.h = __ldg((const unsigned int *)p);
    }
    return u.v;
}

template <typename V, typename I, int KC>
__global__ void __launch_bounds__(RB_THREADS)
grouped_kernel(const gsa_group_item *__restrict__ items, int64_t count, int64_t ntiles, int base,
               int g1_avg, int x_pairs, const int32_t *__restrict__ tile_item) {
    // Each warp finds its tile's item on its own -- lane 0 searches forward from the
    // warp's previous item (a CTA's tiles ascend), the warp reads the item's fields with
    // uniform loads -- so warps never wait for one another between tiles.
    const int lane = threadIdx.x & 31;
    int64_t lo = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        if (tile_item) {  // a batch's table: the tile's item in one load
            lo = __ldg(tile_item + t);
        } else if (lane == 0 && lo + 1 < count && __ldg(&items[lo + 1].first_tile) <= t) {
            int64_t l = lo + 1, h = count - 1;  // last item with first_tile <= t, in (lo, count)
            while (l < h) {
                const int64_t mid = (l + h + 1) >> 1;
                if (__ldg(&items[mid].first_tile) <= t) l = mid;
                else h = mid - 1;
            }
            lo = l;
        }
        if (!tile_item) lo = __shfl_sync(0xffffffffu, lo, 0);
        const gsa_group_item *it = items + lo;
        const int64_t kk = __ldg(&it->k);
        const int64_t ncg = (kk + KC - 1) / KC;
        const int64_t local = t - __ldg(&it->first_tile);
        const int64_t cg = ncg == 1 ? 0 : local % ncg;
        const int64_t unit = ncg == 1 ? local : local / ncg;
        CompressedArgs<V, I> a;
        a.outer_n = __ldg(&it->m);
        a.inner_n = __ldg(&it->n);
        a.nnz = __ldg(&it->nnz);
        a.ptr = (const I *)__ldg((const unsigned long long *)&it->rowptr);
        a.idx = (const I *)__ldg((const unsigned long long *)&it->colval);
        a.val = (const V *)__ldg((const unsigned long long *)&it->nzval);
        a.base = base;
        a.conjA = false;
        const int64_t ldb = __ldg(&it->ldb);
        const bool brow = __ldg(&it->b_rowmajor) != 0;
        DenseIn<V> B;
        B.p = (const V *)__ldg((const unsigned long long *)&it->B);
        B.rs = brow ? ldb : 1;
        B.cs = brow ? 1 : ldb;
        B.conj = false;
        B.pairs = KC >= 2 && x_pairs && std::is_same<V, double>::value && brow && (ldb & 1) == 0 &&
                  ((uintptr_t)B.p & 15) == 0;
        DenseOut<V> C;
        C.p = (V *)__ldg((const unsigned long long *)&it->C);
        C.ld = __ldg(&it->ldc);
        C.alpha = scalar_at<V>(it->alpha);
        C.beta = scalar_at<V>(it->beta);
        C.beta_mode = is_zero(C.beta) ? 0 : (is_one(C.beta) ? 1 : 2);
        C.alpha_one = alpha_one_of(C.alpha);
        const int64_t bin_warps = __ldg(&it->bin_warps);
        if (bin_warps > 0) {  // the plan's bin order: warp w of it
            const int64_t w = unit * RB_WARPS + (threadIdx.x >> 5);
            if (w < bin_warps) {
                const gsa_bin_order *bo = (const gsa_bin_order *)__ldg((const unsigned long long *)&it->bin_order);
                const gsa_bin_order bv{__ldg(&bo->nwarps),
                                       (const int32_t *)__ldg((const unsigned long long *)&bo->perm),
                                       (const int32_t *)__ldg((const unsigned long long *)&bo->warp_group),
                                       (const int64_t *)__ldg((const unsigned long long *)&bo->groups)};
                binned_warp<V, I, KC>(a, kk, B, C, cg * KC, w, bv);
            }
        } else {
            warp_unit<V, I, KC>(a, kk, B, C, cg * KC, unit * RB_THREADS + (threadIdx.x & ~31), nullptr, g1_avg);
        }
    }
}

int default_columns(int dtype) { return dtype_size(dtype) == 8 ? 2 : 4; }  // column-major B

struct GroupedBody {
    cudaStream_t s; const gsa_group_item *items; int64_t count, ntiles; int base, KC, g1;
    const int32_t *tile_item;
    template <typename V, typename I> int operator()() {
        if (ntiles == 0) return GSA_OK;
        auto kern = KC == 1 ? grouped_kernel<V, I, 1>
                  : KC == 2 ? grouped_kernel<V, I, 2>
                  : KC == 4 ? grouped_kernel<V, I, 4> : grouped_kernel<V, I, 8>;
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RB_THREADS, 0),
                            "grouped occupancy");
        if (rc) return rc;
        int64_t grid = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
        if (grid > ntiles) grid = ntiles;
        timer_before(s);
        kern<<<(unsigned)grid, RB_THREADS, 0, s>>>(items, count, ntiles, base, g1, get_x_pairs(), tile_item);
        timer_after(s);
        return check_cuda(cudaGetLastError(), "grouped_kernel");
    }
};

int grouped_mul(cudaStream_t s, int dtype, int itype, int base, const gsa_group_item *d_items,
                int64_t count, int64_t ntiles, int columns, int g1, const int32_t *tile_item = nullptr) {
    // one right-hand side everywhere runs KC = 1; otherwise the batch's KC
    const int KC = columns > 0 ? columns : default_columns(dtype);
    GroupedBody body{s, d_items, count, ntiles, base, KC, g1 > 0 ? g1 : G1_AVG, tile_item};
    return dispatch_vi(dtype, itype, body);
}

}  // namespace gsa

using namespace gsa;

// A batch: items kept on the device (and on the host for the per-call mode), tiles
// counted once with a tile -> item table (so a warp finds its tile's item in one load instead
// of a search), an optional captured graph of the grouped launch.
struct gsa_batch {
    int dtype = 0, itype = 0, base = 1, columns = 0, g1 = 0;
    std::vector<gsa_group_item> host;
    gsa_group_item *dev = nullptr;
    int32_t *tiles = nullptr;
    int64_t ntiles = 0;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

int gsa_grouped_tiles(int dtype, gsa_group_item *items, int64_t count, int columns, int64_t *ntiles) {
    if (!dtype_size(dtype)) return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d", dtype);
    if (!items || count < 0 || !ntiles) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if (columns != 0 && columns != 1 && columns != 2 && columns != 4 && columns != 8)
        return fail(GSA_ERR_INVALID_ARG, "columns must be 0, 1, 2, 4 or 8");
    for (int64_t i = 0; i < count; ++i) {
        const gsa_group_item &it = items[i];
        if (it.m < 0 || it.n < 0 || it.nnz < 0 || it.k < 0)
            return fail(GSA_ERR_INVALID_ARG, "item %lld: negative size", (long long)i);
        const int64_t need_ldb = it.b_rowmajor ? it.k : it.n;
        if (it.b_rowmajor != 0 && it.b_rowmajor != 1)
            return fail(GSA_ERR_INVALID_ARG, "item %lld: b_rowmajor must be 0 or 1", (long long)i);
        if (it.ldb < (need_ldb > 1 ? need_ldb : 1) || it.ldc < (it.m > 1 ? it.m : 1))
            return fail(GSA_ERR_DIM, "item %lld: leading dimension too small", (long long)i);
        if (it.m > 0 && (!it.rowptr || (it.nnz > 0 && (!it.colval || !it.nzval))))
            return fail(GSA_ERR_INVALID_ARG, "item %lld: NULL sparse array", (long long)i);
        if (it.m > 0 && it.k > 0 && (!it.C || (it.n > 0 && !it.B)))
            return fail(GSA_ERR_INVALID_ARG, "item %lld: NULL dense operand", (long long)i);
        if (it.bin_warps < 0 || (it.bin_warps > 0) != (it.bin_order != nullptr))
            return fail(GSA_ERR_INVALID_ARG, "item %lld: bin_order and bin_warps disagree", (long long)i);
    }
    // one column group width for the whole launch: k == 1 items still use KC-wide groups
    // in the kernel, so every item with k > 1 and k == 1 gets ceil(k / KC) groups
    const int KC = columns > 0 ? columns : default_columns(dtype);
    int64_t t = 0;
    for (int64_t i = 0; i < count; ++i) {
        items[i].first_tile = t;
        if (items[i].m > 0 && items[i].k > 0) {
            const int64_t units = items[i].bin_warps > 0 ? ceil_div(items[i].bin_warps, RB_WARPS)
                                                         : ceil_div(items[i].m, RB_THREADS);
            t += units * ceil_div(items[i].k, KC);
        }
    }
    *ntiles = t;
    return GSA_OK;
}

int gsa_grouped_mul(void *stream, int dtype, int itype, int base, const gsa_group_item *d_items,
                    int64_t count, int64_t ntiles, int columns, int g1_avg) {
    if (!dtype_size(dtype) || !itype_size(itype))
        return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (count < 0 || ntiles < 0 || (count > 0 && !d_items)) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    if ((uintptr_t)d_items % 8) return fail(GSA_ERR_INVALID_ARG, "items must be 8-byte aligned");
    if (columns != 0 && columns != 1 && columns != 2 && columns != 4 && columns != 8)
        return fail(GSA_ERR_INVALID_ARG, "columns must be 0, 1, 2, 4 or 8");
    if (count == 0) return GSA_OK;
    return grouped_mul((cudaStream_t)stream, dtype, itype, base, d_items, count, ntiles, columns, g1_avg);
}

int gsa_batch_create(void *stream, int dtype, int itype, int base, const gsa_group_item *items,
                     int64_t count, int columns, int g1_avg, gsa_batch **out) {
    if (!out) return fail(GSA_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!dtype_size(dtype) || !itype_size(itype))
        return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
    if (count < 0 || (count > 0 && !items)) return fail(GSA_ERR_INVALID_ARG, "bad arguments");
    gsa_batch *b = new (std::nothrow) gsa_batch();
    if (!b) return fail(GSA_ERR_ALLOC, "batch: host memory");
    b->dtype = dtype;
    b->itype = itype;
    b->base = base;
    b->columns = columns;
    b->g1 = g1_avg;
    b->host.assign(items, items + count);
    for (int64_t i = 0; itype == GSA_IDX32 && i < count; ++i)
        if (items[i].nnz > 0x7fffffffLL) {
            delete b;
            return fail(GSA_ERR_INVALID_ARG, "item %lld: nnz exceeds what Int32 indices can address",
                        (long long)i);
        }
    int rc = gsa_grouped_tiles(dtype, b->host.data(), count, columns, &b->ntiles);
    if (!rc && count > 0x7fffffffLL) rc = fail(GSA_ERR_UNSUPPORTED, "batch: more than 2^31 - 1 items");
    std::vector<int32_t> table;
    if (!rc && count > 0) {
        table.resize((size_t)b->ntiles);
        for (int64_t i = 0; i < count; ++i) {
            const int64_t t1 = i + 1 < count ? b->host[(size_t)i + 1].first_tile : b->ntiles;
            for (int64_t t = b->host[(size_t)i].first_tile; t < t1; ++t) table[(size_t)t] = (int32_t)i;
        }
        rc = check_cuda(cudaMalloc(&b->dev, sizeof(gsa_group_item) * count), "batch: device items");
        if (!rc && b->ntiles > 0) rc = check_cuda(cudaMalloc(&b->tiles, sizeof(int32_t) * b->ntiles), "batch: tiles");
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(b->dev, b->host.data(), sizeof(gsa_group_item) * count,
                                            cudaMemcpyHostToDevice, (cudaStream_t)stream),
                            "batch: item upload");
        if (!rc && b->ntiles > 0)
            rc = check_cuda(cudaMemcpyAsync(b->tiles, table.data(), sizeof(int32_t) * b->ntiles,
                                            cudaMemcpyHostToDevice, (cudaStream_t)stream),
                            "batch: tile upload");
        if (!rc) rc = check_cuda(cudaStreamSynchronize((cudaStream_t)stream), "batch: sync");
    }
    if (rc) {
        if (b->dev) cudaFree(b->dev);
        if (b->tiles) cudaFree(b->tiles);
        delete b;
        return rc;
    }
    *out = b;
    return GSA_OK;
}

int gsa_batch_run(gsa_batch *b, void *stream, int mode) {
    if (!b) return fail(GSA_ERR_INVALID_ARG, "batch is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t count = (int64_t)b->host.size();
    if (mode == GSA_BATCH_GROUPED)
        return grouped_mul(s, b->dtype, b->itype, b->base, b->dev, count, b->ntiles, b->columns, b->g1, b->tiles);
    if (mode == GSA_BATCH_GRAPH) {
        if (!b->exec) {
            int rc = check_cuda(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "batch: stream");
            if (rc) return rc;
            rc = check_cuda(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "batch: capture");
            if (rc) return rc;
            const int lrc = grouped_mul(b->capture, b->dtype, b->itype, b->base, b->dev, count, b->ntiles,
                                        b->columns, b->g1, b->tiles);
            rc = check_cuda(cudaStreamEndCapture(b->capture, &b->graph), "batch: end capture");
            if (lrc) return lrc;
            if (rc) return rc;
            rc = check_cuda(cudaGraphInstantiate(&b->exec, b->graph, 0), "batch: instantiate");
            if (rc) return rc;
        }
        return check_cuda(cudaGraphLaunch(b->exec, s), "batch: graph launch");
    }
    if (mode == GSA_BATCH_PER_CALL) {
        // one plain product per item, as a loop of gsa_csr_mul calls would issue
        for (int64_t i = 0; i < count; ++i) {
            const gsa_group_item &it = b->host[i];
            const int rc = gsa_csr_mul(stream, b->dtype, b->itype, it.m, it.n, it.nnz, it.rowptr, it.colval,
                                       it.nzval, b->base, GSA_OP_N, it.k, it.B, it.ldb,
                                       it.b_rowmajor ? GSA_OP_T : GSA_OP_N, it.C,
                                       it.ldc, it.alpha, it.beta, GSA_ALGO_AUTO, nullptr, 0);
            if (rc) return rc;
        }
        return GSA_OK;
    }
    return fail(GSA_ERR_INVALID_ARG, "unknown batch mode %d", mode);
}

int gsa_batch_destroy(gsa_batch *b) {
    if (!b) return GSA_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture) cudaStreamDestroy(b->capture);
    int rc = b->dev ? check_cuda(cudaFree(b->dev), "batch: free") : GSA_OK;
    if (b->tiles) {
        const int rc2 = check_cuda(cudaFree(b->tiles), "batch: free");
        rc = rc ? rc : rc2;
    }
    delete b;
    return rc;
}

}  // extern "C"
