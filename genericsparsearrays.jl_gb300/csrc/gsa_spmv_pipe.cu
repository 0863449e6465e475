// Persistent, bulk-copy-pipelined row-gather SpMV (one right-hand side):
//   y[o] = beta*y[o] + alpha * sum_j a_j * x[idx_j]
// over the compressed outer dimension -- the work of kernel_spmatmul_csr_N!
// (src/matrix_csr/matrix_csr_kernels.jl:1-22) and kernel_spmatmul_csc_T!
// (src/matrix_csc/matrix_csc_kernels.jl:24-45) for a vector x.
//
// Work split: the merge path of the outer end offsets and the stored entries
// (Merrill & Garland, SC'16) is cut into tiles of TILE items (an item is one
// stored entry or one row end), and every CTA owns one contiguous run of tiles,
// so CTAs get equal numbers of items whatever the row-length mix.
//
// Per CTA:
//   * one cooperative search of the pointer array (THREADS-ary) finds the start
//     of its run; after that each tile's end comes from a 2*THREADS-row probe of
//     the pointer array, with no separate partition pass
//   * the index and value streams of the NEXT tile are copied into shared
//     memory by the bulk-copy engine (cp.async.bulk + mbarrier, 16-byte aligned
//     interior; the <16-byte head and tail by plain loads) while the current
//     tile is reduced, so HBM streaming overlaps the x gathers
//   * phase 1 (balanced over entries): every thread forms the products
//     a_j * x[idx_j] of TILE/THREADS entries, all gathers in flight together,
//     and writes them over the staged values
//   * phase 2 (over rows): a thread sums a row portion of <= 32 products, a
//     warp one of <= 1024, the whole CTA a longer one; every order is fixed, so
//     results are deterministic
//   * the partial of a row that continues into the next tile is carried in
//     shared memory; only the open row at the end of a CTA's run goes to the
//     fixup pass, in CTA order (no atomics)
// Every mbarrier wait is bounded; a wait that gives up sets the device error
// word (read by gsa_check_device_status) and the CTA returns.
#include <atomic>
#include <mutex>

#include "gsa_internal.cuh"

namespace gsa {

__device__ int g_pipe_error = 0;

constexpr int SHORT_ROW = 32;               // thread-per-row limit
constexpr int WARP_ROW = 1024;              // warp-per-row limit
constexpr uint32_t WAIT_LIMIT = 1u << 24;   // bounded mbarrier polls (default)
// Polls before a tile's wait gives up (gsa_set_tuning(GSA_TUNE_WAIT_LIMIT); a small value
// makes the timeout path run).  Draining copies after a give-up always uses WAIT_LIMIT.
static std::atomic<uint32_t> g_wait_limit{WAIT_LIMIT};
void set_wait_limit(uint32_t polls) { g_wait_limit.store(polls, std::memory_order_relaxed); }
uint32_t get_wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }

template <typename V> struct PipeShape {
    static constexpr int TILE = sizeof(V) >= 16 ? 1024 : 2048;
};

// ---- PTX helpers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// One array segment [a, b) of a stream, placed so that its 16-byte-aligned
// interior lands on 16-byte-aligned shared memory.
struct Segment {
    uintptr_t ga, gb;      // global byte range
    uintptr_t lo16, hi16;  // aligned interior (valid when hi16 > lo16)
    __device__ __forceinline__ Segment(const void *base, int64_t a, int64_t b, int esize) {
        ga = (uintptr_t)base + (uintptr_t)(a * esize);
        gb = (uintptr_t)base + (uintptr_t)(b * esize);
        lo16 = (ga + 15) & ~(uintptr_t)15;
        hi16 = gb & ~(uintptr_t)15;
    }
    __device__ __forceinline__ bool has_interior() const { return hi16 > lo16; }
    __device__ __forceinline__ uint32_t interior_bytes() const {
        return has_interior() ? (uint32_t)(hi16 - lo16) : 0u;
    }
    // shared-memory address of global byte g for a stage buffer at sbuf
    __device__ __forceinline__ unsigned char *map(unsigned char *sbuf, uintptr_t g) const {
        return sbuf + (g - (ga & ~(uintptr_t)15));
    }
};

template <typename V, typename I, int THREADS> struct PipeSmem {
    static constexpr int TILE = PipeShape<V>::TILE;
    static constexpr int WARPS = THREADS / 32;
    static constexpr int LONG_CAP = TILE / (SHORT_ROW + 1) + 2;
    alignas(16) unsigned char col[2][TILE * sizeof(I) + 16];
    alignas(16) unsigned char val[2][TILE * sizeof(V) + 16];
    int rowend[TILE];
    V red[WARPS];
    V carry[2];
    uint64_t bar[2];
    int nlong;
    int huge;
    int longrow[LONG_CAP];
};

// First r in [lo, hi) with end(r) + r >= D (hi if none): a THREADS-ary search,
// one pointer load per thread per round.  Uniform across the CTA.
template <typename I, int THREADS>
__device__ int64_t coop_search(const I *__restrict__ ptr, int base, int64_t lo, int64_t hi, int64_t D) {
    while (lo < hi) {
        const int64_t step = (hi - lo + THREADS - 1) / THREADS;
        const int64_t p = lo + (int64_t)threadIdx.x * step;
        const bool f = p < hi && ((int64_t)__ldg(ptr + p + 1) - base + p < D);
        const int c = __syncthreads_count(f);
        const int64_t nlo = c > 0 ? lo + (int64_t)(c - 1) * step + 1 : lo;
        const int64_t nhi = lo + (int64_t)c * step;
        hi = nhi < hi ? nhi : hi;
        lo = nlo;
    }
    return lo;
}

// x[col] (conjugated if op(B) is an adjoint); indices outside [0, inner_n) read nothing.
template <typename V, typename I>
__device__ __forceinline__ V load_x(const CompressedArgs<V, I> &a, const DenseIn<V> &B, I col) {
    if (sizeof(I) == 4) {  // Int32 indices: inner_n < 2^31, 32-bit index math
        const int ci = (int)col - a.base;
        if ((unsigned)ci >= (unsigned)a.inner_n) return VT<V>::zero();
        return conj_if(ldg(B.p + (int64_t)ci * B.rs), B.conj);
    }
    const int64_t ci = (int64_t)col - a.base;
    if ((uint64_t)ci >= (uint64_t)a.inner_n) return VT<V>::zero();
    return conj_if(ldg(B.p + ci * B.rs), B.conj);
}

// Resident CTAs per SM the register cap is sized for: three 256-thread CTAs
// (their shared memory fits three times), or two 512-thread CTAs.
template <typename V, typename I, int THREADS>
__global__ void __launch_bounds__(THREADS, THREADS >= 512 ? 2 : 3)
spmv_pipe_kernel(CompressedArgs<V, I> a, DenseIn<V> B, DenseOut<V> C, int64_t tiles_per_cta,
                 int64_t *__restrict__ carry_row, V *__restrict__ carry_val, uint32_t wait_limit) {
    using S_t = PipeSmem<V, I, THREADS>;
    constexpr int TILE = S_t::TILE;
    constexpr int WARPS = S_t::WARPS;
    constexpr int LONG_CAP = S_t::LONG_CAP;
    constexpr int PROBE = 2 * THREADS;
    constexpr int U = TILE / THREADS;  // entries per thread in phase 1
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S_t &S = *reinterpret_cast<S_t *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t total = a.outer_n + a.nnz;
    const int64_t D0 = (int64_t)blockIdx.x * tiles_per_cta * TILE;
    if (D0 >= total) {
        if (tid == 0) carry_row[blockIdx.x] = -1;
        return;
    }
    const int64_t Dend = D0 + tiles_per_cta * TILE < total ? D0 + tiles_per_cta * TILE : total;
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_mbar_init();
        S.carry[0] = VT<V>::zero();
    }
    // start of this CTA's run on diagonal D0
    int64_t rs = coop_search<I, THREADS>(a.ptr, a.base, D0 - a.nnz > 0 ? D0 - a.nnz : 0,
                                         D0 < a.outer_n ? D0 : a.outer_n, D0);
    int64_t js = D0 - rs;

    uint32_t inflight = 0u;  // bit st: stage st has copies not yet waited for (thread 0's view)
    // copies of [j0, min(j0 + TILE, nnz)) into stage st
    auto issue = [&](int st, int64_t j0) {
        j0 = j0 < 0 ? 0 : (j0 > a.nnz ? a.nnz : j0);
        const int64_t j1 = j0 + TILE < a.nnz ? j0 + TILE : a.nnz;
        const Segment sc(a.idx, j0, j1, sizeof(I)), sv(a.val, j0, j1, sizeof(V));
        if (tid == 0) {
            inflight |= 1u << st;
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(&S.bar[st], sc.interior_bytes() + sv.interior_bytes());
            if (sc.has_interior())
                bulk_copy_g2s(sc.map(S.col[st], sc.lo16), (const void *)sc.lo16, sc.interior_bytes(), &S.bar[st]);
            if (sv.has_interior())
                bulk_copy_g2s(sv.map(S.val[st], sv.lo16), (const void *)sv.lo16, sv.interior_bytes(), &S.bar[st]);
        } else if (tid >= 32 && tid < 64) {
            // head and tail (fewer than 16 bytes each) by plain loads
            const bool col_side = tid < 48;
            const Segment &sg = col_side ? sc : sv;
            const int es = col_side ? (int)sizeof(I) : (int)sizeof(V);
            const int k = tid & 15;  // element slot: 0..3 head, 4..7 tail
            uintptr_t g = 0;
            bool ok = false;
            if (sg.has_interior()) {
                if (k < 4) { g = sg.ga + (uintptr_t)k * es; ok = g < sg.lo16; }
                else if (k < 8) { g = sg.hi16 + (uintptr_t)(k - 4) * es; ok = g < sg.gb; }
            } else {
                g = sg.ga + (uintptr_t)k * es;
                ok = k < 8 && g < sg.gb;
            }
            if (ok) {
                unsigned char *d = sg.map(col_side ? S.col[st] : S.val[st], g);
                if (col_side) *reinterpret_cast<I *>(d) = ld_stream(reinterpret_cast<const I *>(g));
                else *reinterpret_cast<V *>(d) = ld_stream(reinterpret_cast<const V *>(g));
            }
        }
    };

    // probe: end offsets of rows r0 + tid and r0 + THREADS + tid
    int64_t pe0, pe1;
    auto probe = [&](int64_t r0) {
        const int64_t r_a = r0 + tid, r_b = r0 + THREADS + tid;
        pe0 = r_a < a.outer_n ? (int64_t)__ldg(a.ptr + r_a + 1) - a.base : INT64_MAX / 2;
        pe1 = r_b < a.outer_n ? (int64_t)__ldg(a.ptr + r_b + 1) - a.base : INT64_MAX / 2;
    };

    probe(rs);
    issue(0, js);
    uint32_t parity = 0u;  // bit st: phase parity of stage st
    bool failed = false;
    int64_t d0 = D0;
    int64_t re = rs;
    int it = 0;
    for (; d0 < Dend; ++it) {
        const int st = it & 1;
        const int64_t d1 = d0 + TILE < Dend ? d0 + TILE : Dend;
        // ---- end coordinate of this tile
        const bool f0 = pe0 + (rs + tid) < d1;
        const bool f1 = pe1 + (rs + THREADS + tid) < d1;
        int cnt = __syncthreads_count(f0);
        if (cnt == THREADS) cnt += __syncthreads_count(f1);
        if (cnt == PROBE) {
            const int64_t lo = rs + PROBE > d1 - a.nnz ? rs + PROBE : d1 - a.nnz;
            re = coop_search<I, THREADS>(a.ptr, a.base, lo, d1 < a.outer_n ? d1 : a.outer_n, d1);
        } else {
            re = rs + cnt;
        }
        re = re < rs ? rs : (re > a.outer_n ? a.outer_n : re);
        const int64_t je = d1 - re;
        // a malformed pointer array can only make a tile wrong, never out of bounds
        int tile_rows = (int)(re - rs), tile_nnz = (int)(je - js);
        if (tile_rows > TILE || tile_nnz < 0 || tile_nnz > TILE || js < 0 || je > a.nnz)
            tile_rows = tile_nnz = 0;
        auto local_end = [&](int64_t end) {
            const int64_t v = end - js;
            return (int)(v < 0 ? 0 : (v > tile_nnz ? tile_nnz : v));
        };
        if (tid < tile_rows) S.rowend[tid] = local_end(pe0);
        if (THREADS + tid < tile_rows) S.rowend[THREADS + tid] = local_end(pe1);
        for (int e = PROBE + tid; e < tile_rows; e += THREADS)
            S.rowend[e] = local_end((int64_t)__ldg(a.ptr + rs + 1 + e) - a.base);
        if (tid == 0) { S.nlong = 0; S.huge = -1; }
        // ---- prefetch the next tile
        if (d1 < Dend) {
            probe(re);
            issue(st ^ 1, je);
        }
        // ---- wait for this tile's streams
        bool ok = false;
        for (uint32_t w = 0; w < wait_limit; ++w)
            if ((ok = mbar_try_wait(&S.bar[st], (parity >> st) & 1u))) break;
        if (ok) {
            parity ^= 1u << st;
            inflight &= ~(1u << st);
        }
        if (__syncthreads_or(!ok)) { failed = true; break; }

        const Segment sc(a.idx, js, js, sizeof(I)), sv(a.val, js, js, sizeof(V));
        const I *tcol = reinterpret_cast<const I *>(sc.map(S.col[st], sc.ga));
        V *tv = reinterpret_cast<V *>(sv.map(S.val[st], sv.ga));

        // ---- phase 1: products of all entries, gathers in flight together
        {
            I cj[U];
            V av[U], xv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = tid + u * THREADS;
                if (e < tile_nnz) { cj[u] = tcol[e]; av[u] = tv[e]; }
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (tid + u * THREADS < tile_nnz) xv[u] = load_x<V, I>(a, B, cj[u]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int e = tid + u * THREADS;
                if (e < tile_nnz) tv[e] = mul(conj_if(av[u], a.conjA), xv[u]);
            }
        }
        __syncthreads();

        // ---- phase 2: row sums over the products
        const V carry_in = S.carry[st];
        const int last = re < a.outer_n ? tile_rows : tile_rows - 1;  // the open row too
        for (int e = tid; e <= last; e += THREADS) {
            const int b0 = e == 0 ? 0 : S.rowend[e - 1];
            const int b1 = e < tile_rows ? S.rowend[e] : tile_nnz;
            const int len = b1 - b0;
            if (len > WARP_ROW) { S.huge = e; continue; }
            if (len > SHORT_ROW) {
                const int q = atomicAdd(&S.nlong, 1);
                if (q < LONG_CAP) S.longrow[q] = e;
                continue;
            }
            V acc = VT<V>::zero();
            for (int j = b0; j < b1; ++j) acc = add(acc, tv[j]);
            if (e == 0) acc = add(carry_in, acc);
            if (e < tile_rows) C.store(rs + e, 0, acc);
            else S.carry[st ^ 1] = acc;
        }
        __syncthreads();
        // portions of 33..1024 entries: a warp each
        const int nlong = S.nlong < LONG_CAP ? S.nlong : LONG_CAP;
        for (int q = warp; q < nlong; q += WARPS) {
            const int e = S.longrow[q];
            const int b0 = e == 0 ? 0 : S.rowend[e - 1];
            const int b1 = e < tile_rows ? S.rowend[e] : tile_nnz;
            V acc = VT<V>::zero();
            for (int j = b0 + lane; j < b1; j += 32) acc = add(acc, tv[j]);
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) acc = add(acc, shfl_xor(acc, m));
            if (lane == 0) {
                if (e == 0) acc = add(carry_in, acc);
                if (e < tile_rows) C.store(rs + e, 0, acc);
                else S.carry[st ^ 1] = acc;
            }
        }
        // one portion of more than 1024 entries: the whole CTA
        const int huge = S.huge;
        if (huge >= 0) {
            const int e = huge;
            const int b0 = e == 0 ? 0 : S.rowend[e - 1];
            const int b1 = e < tile_rows ? S.rowend[e] : tile_nnz;
            V acc = VT<V>::zero();
            for (int j = b0 + tid; j < b1; j += THREADS) acc = add(acc, tv[j]);
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) acc = add(acc, shfl_xor(acc, m));
            if (lane == 0) S.red[warp] = acc;
            __syncthreads();
            if (tid == 0) {
                V t = S.red[0];
                for (int w = 1; w < WARPS; ++w) t = add(t, S.red[w]);
                if (e == 0) t = add(carry_in, t);
                if (e < tile_rows) C.store(rs + e, 0, t);
                else S.carry[st ^ 1] = t;
            }
        }
        __syncthreads();
        rs = re;
        js = je;
        d0 = d1;
    }
    if (failed) {
        // let copies still in flight land before the CTA's shared memory goes away (the
        // stages thread 0 issued and has not seen complete; the default bound, whatever
        // the tile waits used)
        if (tid == 0) {
            atomicOr(&g_pipe_error, 1);
            for (int st = 0; st < 2; ++st) {
                if (!((inflight >> st) & 1u)) continue;
                for (uint32_t w = 0; w < WAIT_LIMIT; ++w)
                    if (mbar_try_wait(&S.bar[st], (parity >> st) & 1u)) break;
            }
            carry_row[blockIdx.x] = -1;
        }
        return;
    }
    if (tid == 0) {
        // the row left open at the end of the run (completed by a later CTA)
        const bool open = re < a.outer_n;
        carry_row[blockIdx.x] = open ? re : -1;
        carry_val[blockIdx.x] = open ? S.carry[it & 1] : VT<V>::zero();
    }
}

// One entry per CTA; runs of CTAs carrying one row are summed in CTA order.
template <typename V>
__global__ void pipe_fixup_kernel(int64_t n, const int64_t *__restrict__ carry_row,
                                  const V *__restrict__ carry_val, DenseOut<V> C) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int64_t r = carry_row[t];
    if (r < 0 || (t > 0 && carry_row[t - 1] == r)) return;
    V sum = carry_val[t];
    for (int64_t t2 = t + 1; t2 < n && carry_row[t2] == r; ++t2) sum = add(sum, carry_val[t2]);
    C.accumulate(r, 0, mul(sum, C.alpha));
}

// Threads per CTA of the pipelined kernel (256 or 512); settable for tuning from any host
// thread, so an atomic read once per launch.
static std::atomic<int> g_pipe_threads{512};
void set_pipe_threads(int t) { g_pipe_threads.store(t == 256 ? 256 : 512, std::memory_order_relaxed); }
int get_pipe_threads() { return g_pipe_threads.load(std::memory_order_relaxed); }

template <typename V, typename I>
size_t spmv_pipe_workspace_size(int64_t outer_n, int64_t nnz) {
    const int64_t T = ceil_div(outer_n + nnz, PipeShape<V>::TILE);
    Carver cv(nullptr);
    cv.take<int64_t>(T);
    cv.take<V>(T);
    return align_up(cv.off, 256);
}

template <typename V, typename I, int THREADS>
static int launch_pipe_impl(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B,
                            DenseOut<V> C, void *ws, size_t ws_bytes) {
    constexpr int TILE = PipeShape<V>::TILE;
    const size_t smem = sizeof(PipeSmem<V, I, THREADS>);
    auto kern = spmv_pipe_kernel<V, I, THREADS>;
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "spmv_pipe smem attribute");
    if (rc) return rc;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem),
                    "spmv_pipe occupancy");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    const int64_t T = ceil_div(a.outer_n + a.nnz, TILE);
    int64_t G = (int64_t)sms * per_sm;
    if (G > T) G = T;
    const int64_t Q = ceil_div(T, G);
    G = ceil_div(T, Q);
    if (ws_bytes < spmv_pipe_workspace_size<V, I>(a.outer_n, a.nnz))
        return fail(GSA_ERR_INVALID_ARG, "spmv workspace too small");
    Carver cv(ws);
    int64_t *carry_row = cv.take<int64_t>(T);
    V *carry_val = cv.take<V>(T);
    timer_before(s);
    kern<<<(unsigned)G, THREADS, smem, s>>>(a, B, C, Q, carry_row, carry_val, get_wait_limit());
    timer_after(s);
    rc = check_cuda(cudaGetLastError(), "spmv_pipe_kernel");
    if (rc) return rc;
    pipe_fixup_kernel<V><<<(unsigned)ceil_div(G, 256), 256, 0, s>>>(G, carry_row, carry_val, C);
    return check_cuda(cudaGetLastError(), "pipe_fixup_kernel");
}

template <typename V, typename I>
int launch_spmv_pipe(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B, DenseOut<V> C,
                     void *ws, size_t ws_bytes) {
    if (a.outer_n == 0) return GSA_OK;
    if (get_pipe_threads() == 256) return launch_pipe_impl<V, I, 256>(s, a, B, C, ws, ws_bytes);
    return launch_pipe_impl<V, I, 512>(s, a, B, C, ws, ws_bytes);
}

// ---------------------------------------------------------------------------
// SpMV without any allocation (gsa_csr_spmv_noalloc).
//
// Some callers cannot allocate device memory at the moment they need a
// product: a process whose device memory is already owned by another pool (so
// cudaMalloc fails), or code that must not let an allocation synchronize the
// device or, in Julia, run the garbage collector and its finalizers.  For them
// the carry slots of the pipelined kernel -- its only scratch -- live in this
// file-scope device array instead of a workspace.  The array is part of the
// library's device image: every GPU that loads the library's kernels holds it
// (NOALLOC_MAX_RUNS * 24 bytes = 192 KiB) until the process exits.  It is shared
// by every call, so calls that overlap on the GPU race on it.  No slot has to
// start at zero: each slot the fixup reads is written earlier in the same call.
constexpr int64_t NOALLOC_MAX_RUNS = 8192;  // CTA runs (= carry slots) per call
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_MAX_RUNS * (8 + 16)];

// Device address of g_noalloc_scratch on the current device, looked up once per
// device (the first call on a device does this set-up).
static int noalloc_scratch(unsigned char **out) {
    static std::mutex mu;
    static void *addr[128] = {};
    int dev = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "noalloc: current device");
    if (rc) return rc;
    if (dev < 0 || dev >= 128) return fail(GSA_ERR_UNSUPPORTED, "noalloc: device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "noalloc: scratch address");
        if (rc) return rc;
        addr[dev] = p;
    }
    *out = (unsigned char *)addr[dev];
    return GSA_OK;
}

template <typename V, typename I, int THREADS>
static int launch_noalloc_impl(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B,
                               DenseOut<V> C) {
    constexpr int TILE = PipeShape<V>::TILE;
    const size_t smem = sizeof(PipeSmem<V, I, THREADS>);
    auto kern = spmv_pipe_kernel<V, I, THREADS>;
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "spmv_pipe smem attribute");
    if (rc) return rc;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem),
                    "spmv_pipe occupancy");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    const int64_t T = ceil_div(a.outer_n + a.nnz, TILE);
    int64_t G = (int64_t)sms * per_sm;
    if (G > T) G = T;
    const int64_t Q = ceil_div(T, G);
    G = ceil_div(T, Q);
    if (G > NOALLOC_MAX_RUNS)
        return fail(GSA_ERR_INVALID_ARG,
                    "noalloc SpMV needs %lld carry slots, more than the %lld of its static scratch",
                    (long long)G, (long long)NOALLOC_MAX_RUNS);
    unsigned char *scratch = nullptr;
    rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    int64_t *carry_row = reinterpret_cast<int64_t *>(scratch);
    V *carry_val = reinterpret_cast<V *>(scratch + NOALLOC_MAX_RUNS * 8);
    kern<<<(unsigned)G, THREADS, smem, s>>>(a, B, C, Q, carry_row, carry_val, get_wait_limit());
    rc = check_cuda(cudaGetLastError(), "spmv_pipe_kernel (noalloc)");
    if (rc) return rc;
    pipe_fixup_kernel<V><<<(unsigned)ceil_div(G, 256), 256, 0, s>>>(G, carry_row, carry_val, C);
    return check_cuda(cudaGetLastError(), "pipe_fixup_kernel (noalloc)");
}

template <typename V, typename I>
int launch_spmv_noalloc(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B, DenseOut<V> C) {
    if (a.outer_n == 0) return GSA_OK;
    if (get_pipe_threads() == 256) return launch_noalloc_impl<V, I, 256>(s, a, B, C);
    return launch_noalloc_impl<V, I, 512>(s, a, B, C);
}

int read_pipe_error(cudaStream_t s, int *out) {
    int rc = check_cuda(cudaStreamSynchronize(s), "device status sync");
    if (rc) return rc;
    int zero = 0;
    rc = check_cuda(cudaMemcpyFromSymbol(out, g_pipe_error, sizeof(int)), "device status read");
    if (rc) return rc;
    return check_cuda(cudaMemcpyToSymbol(g_pipe_error, &zero, sizeof(int)), "device status clear");
}

#define GSA_INST_PIPE(V, I)                                                                     \
    template int launch_spmv_pipe<V, I>(cudaStream_t, const CompressedArgs<V, I> &, DenseIn<V>, \
                                        DenseOut<V>, void *, size_t);                           \
    template size_t spmv_pipe_workspace_size<V, I>(int64_t, int64_t);                           \
    template int launch_spmv_noalloc<V, I>(cudaStream_t, const CompressedArgs<V, I> &,          \
                                           DenseIn<V>, DenseOut<V>);
GSA_INST_PIPE(float, int32_t)
GSA_INST_PIPE(float, int64_t)
GSA_INST_PIPE(double, int32_t)
GSA_INST_PIPE(double, int64_t)
GSA_INST_PIPE(cf32, int32_t)
GSA_INST_PIPE(cf32, int64_t)
GSA_INST_PIPE(cf64, int32_t)
GSA_INST_PIPE(cf64, int64_t)
GSA_INST_PIPE(int32_t, int32_t)
GSA_INST_PIPE(int32_t, int64_t)
GSA_INST_PIPE(int64_t, int32_t)
GSA_INST_PIPE(int64_t, int64_t)

}  // namespace gsa
