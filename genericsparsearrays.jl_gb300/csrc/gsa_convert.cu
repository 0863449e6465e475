// Format conversions.
//
// COO -> CSR / CSC (src/conversions/conversions.jl:171-212,282-323).  The
// reference builds key = major*minor_dim + minor in the index type (wrapping
// for Int32 once major_dim*minor_dim >= 2^31), sortperms the keys with
// AcceleratedKernels, gathers the three arrays and binary-searches every
// major index.  Here the same order (by major, then minor, ties in input order)
// comes from a bucket sort on the major index (gsa_bucket.cuh): a count per
// major index, one scan -- which is the output's pointer array -- a placement of
// (minor << 32 | position) keys into their buckets, and a sort of each bucket on
// its own, whose emitter writes the minor index and gathers the value.  Matrices
// whose sizes do not fit the bucket keys' 32-bit fields take the LSD radix sort:
//   1. make_keys_kernel: key = (major << minor_bits) | minor as an unsigned
//      64-bit word (no multiply, no wrap), payload = the entry's position
//   2. 8-bit digits, only over the key bits that can be set; each pass =
//      per-tile digit histograms, one exclusive scan, a stable scatter (warp
//      match_any ranking in storage order)
//   3. finalize_kernel: minor index straight from the key, value gathered by
//      the payload; pointer_kernel: pointer entries from the boundaries of the
//      sorted major indices (every entry written exactly once)
// Both sorts are stable, so duplicate (row, col) pairs keep input order.
//
// CSR / CSC -> COO (src/conversions/conversion_kernels.jl:2-35): the major
// index of every entry is written by merge-path tiles (balanced for any row
// length mix); minor indices and values are plain copies.
#include <atomic>
#include <type_traits>

#include "gsa_internal.cuh"
#include "gsa_bucket.cuh"

namespace gsa {

static std::atomic<int> g_sort_staged{1};
void set_sort_staged(int v) { g_sort_staged.store(v, std::memory_order_relaxed); }
int get_sort_staged() { return g_sort_staged.load(std::memory_order_relaxed); }

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 8;                       // 32-entry rounds per warp
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;    // entries per tile
constexpr int RS_BITS = 8;
constexpr int RS_BINS = 1 << RS_BITS;

static int bits_for(int64_t count) {  // bits needed for values 0..count-1
    int b = 0;
    while (b < 63 && ((int64_t)1 << b) < count) ++b;
    return b;
}

template <typename I>
__global__ void make_keys_kernel(int64_t nnz, const I *__restrict__ major, const I *__restrict__ minor,
                                 int base, int minor_bits, uint64_t *__restrict__ keys,
                                 uint32_t *__restrict__ perm) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t hi = (uint64_t)((int64_t)ld_stream(major + i) - base);
        uint64_t lo = (uint64_t)((int64_t)ld_stream(minor + i) - base);
        keys[i] = minor_bits >= 64 ? lo : ((hi << minor_bits) | lo);
        perm[i] = (uint32_t)i;
    }
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Per-tile digit histograms, digit-major: hist[d * num_tiles + tile].
__global__ void __launch_bounds__(RS_THREADS)
radix_upsweep_kernel(const uint64_t *__restrict__ keys, int64_t n, int shift, uint32_t mask,
                     uint32_t *__restrict__ hist, int64_t num_tiles) {
    __shared__ uint32_t s_h[RS_BINS];
    const int tid = threadIdx.x, lane = tid & 31;
    for (int d = tid; d < RS_BINS; d += RS_THREADS) s_h[d] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        int64_t e = t0 + (int64_t)r * RS_THREADS + tid;
        uint32_t d = e < n ? (uint32_t)(keys[e] >> shift) & mask : RS_BINS;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        if (d < RS_BINS && lane == __ffs(peers) - 1) atomicAdd(&s_h[d], __popc(peers));
    }
    __syncthreads();
    for (int d = tid; d < RS_BINS; d += RS_THREADS) hist[(int64_t)d * num_tiles + blockIdx.x] = s_h[d];
}

// Stable scatter.  Warp w of a tile owns entries [w*32*ROUNDS, (w+1)*32*ROUNDS) of the
// tile and ranks them round by round; per-warp digit counts give each entry its place in
// the tile sorted by digit.  The tile is first written there, in shared memory, and then
// copied out in that order: consecutive threads write consecutive addresses of one digit's
// run, instead of every lane of a round writing to a different bucket.
__global__ void __launch_bounds__(RS_THREADS)
radix_downsweep_kernel(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ perm_in,
                       uint64_t *__restrict__ keys_out, uint32_t *__restrict__ perm_out, int64_t n,
                       int shift, uint32_t mask, const uint32_t *__restrict__ offsets,
                       int64_t num_tiles) {
    __shared__ uint32_t s_wh[RS_WARPS][RS_BINS];
    __shared__ uint32_t s_toff[RS_BINS];   // first position of each digit in the sorted tile
    __shared__ uint32_t s_goff[RS_BINS];   // its first position in the output
    __shared__ uint64_t s_key[RS_TILE];
    __shared__ uint32_t s_perm[RS_TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int t = tid; t < RS_WARPS * RS_BINS; t += RS_THREADS) (&s_wh[0][0])[t] = 0;
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * RS_TILE;
    const int64_t w0 = tile0 + (int64_t)warp * 32 * RS_ROUNDS;
    const int tile_n = (int)(n - tile0 < RS_TILE ? n - tile0 : RS_TILE);
    const unsigned lt = lanemask_lt();
    uint64_t key[RS_ROUNDS];
    uint32_t pv[RS_ROUNDS], rank[RS_ROUNDS], dig[RS_ROUNDS];
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        int64_t e = w0 + r * 32 + lane;
        bool valid = e < n;
        key[r] = valid ? keys_in[e] : 0;
        pv[r] = valid ? perm_in[e] : 0;
        dig[r] = valid ? (uint32_t)(key[r] >> shift) & mask : RS_BINS;
    }
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        uint32_t d = dig[r];
        unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = d < RS_BINS ? s_wh[warp][d] : 0;
        rank[r] = before + __popc(peers & lt);
        __syncwarp();
        if (d < RS_BINS && lane == __ffs(peers) - 1) s_wh[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit (a thread each, RS_THREADS == RS_BINS): the warps' starts inside the digit's
    // run, the run's size; then an exclusive scan of the sizes gives the runs' tile offsets
    static_assert(RS_THREADS == RS_BINS, "one thread per digit");
    {
        const int d = tid;
        uint32_t run = 0;
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t c = s_wh[w][d];
            s_wh[w][d] = run;
            run += c;
        }
        s_toff[d] = run;  // the size for now
        s_goff[d] = offsets[(int64_t)d * num_tiles + blockIdx.x];
    }
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the 256 run sizes by one warp, 8 per lane
        uint32_t v[RS_BINS / 32], sum = 0;
#pragma unroll
        for (int q = 0; q < RS_BINS / 32; ++q) {
            v[q] = s_toff[lane * (RS_BINS / 32) + q];
            sum += v[q];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int q = 0; q < RS_BINS / 32; ++q) {
            s_toff[lane * (RS_BINS / 32) + q] = run;
            run += v[q];
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        if (dig[r] < RS_BINS) {
            const uint32_t lp = s_toff[dig[r]] + s_wh[warp][dig[r]] + rank[r];
            s_key[lp] = key[r];
            s_perm[lp] = pv[r];
        }
    }
    __syncthreads();
    for (int i = tid; i < tile_n; i += RS_THREADS) {
        const uint64_t k = s_key[i];
        const uint32_t d = (uint32_t)(k >> shift) & mask;
        const uint32_t pos = s_goff[d] + (uint32_t)i - s_toff[d];
        keys_out[pos] = k;
        perm_out[pos] = s_perm[i];
    }
}

// ---- exclusive scan of uint32 counts (reduce, scan of block sums, downsweep)
constexpr int SC_THREADS = 512;
constexpr int SC_ITEMS = 8;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__device__ __forceinline__ uint32_t block_excl_scan_u32(uint32_t v, uint32_t *s_warp, uint32_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W = SC_THREADS / 32;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < W ? s_warp[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= off) s += y;
        }
        if (lane < W) s_warp[lane] = s;
    }
    __syncthreads();
    uint32_t warp_prefix = warp > 0 ? s_warp[warp - 1] : 0;
    total = s_warp[W - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SC_THREADS)
scan_reduce_kernel(const uint32_t *__restrict__ in, int64_t n, uint32_t *__restrict__ block_sums) {
    __shared__ uint32_t s_warp[SC_THREADS / 32];
    const int64_t t0 = (int64_t)blockIdx.x * SC_TILE;
    uint32_t sum = 0;
#pragma unroll
    for (int u = 0; u < SC_ITEMS; ++u) {
        int64_t e = t0 + (int64_t)u * SC_THREADS + threadIdx.x;
        if (e < n) sum += in[e];
    }
    uint32_t total;
    block_excl_scan_u32(sum, s_warp, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Single CTA: exclusive scan of the block sums in place (any count).
__global__ void __launch_bounds__(SC_THREADS)
scan_block_sums_kernel(uint32_t *__restrict__ sums, int64_t nb) {
    __shared__ uint32_t s_warp[SC_THREADS / 32];
    uint32_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += SC_THREADS) {
        int64_t e = b0 + threadIdx.x;
        uint32_t v = e < nb ? sums[e] : 0;
        uint32_t total;
        uint32_t ex = block_excl_scan_u32(v, s_warp, total);
        if (e < nb) sums[e] = carry + ex;
        carry += total;
    }
}

// Each thread scans SC_ITEMS consecutive entries (blocked arrangement).
__global__ void __launch_bounds__(SC_THREADS)
scan_downsweep_kernel(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, int64_t n,
                      const uint32_t *__restrict__ block_prefix) {
    __shared__ uint32_t s_warp[SC_THREADS / 32];
    const int64_t t0 = (int64_t)blockIdx.x * SC_TILE + (int64_t)threadIdx.x * SC_ITEMS;
    uint32_t v[SC_ITEMS], sum = 0;
#pragma unroll
    for (int u = 0; u < SC_ITEMS; ++u) {
        v[u] = t0 + u < n ? in[t0 + u] : 0;
        sum += v[u];
    }
    uint32_t total;
    uint32_t run = block_excl_scan_u32(sum, s_warp, total) + block_prefix[blockIdx.x];
#pragma unroll
    for (int u = 0; u < SC_ITEMS; ++u) {
        if (t0 + u < n) out[t0 + u] = run;
        run += v[u];
    }
}

// The reduce kernel sums each SC_TILE slice in striped order and the downsweep
// scans the same slice in blocked order: both cover [b*SC_TILE, (b+1)*SC_TILE).
static int exclusive_scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n,
                              uint32_t *block_sums) {
    if (n == 0) return GSA_OK;
    int64_t nb = ceil_div(n, SC_TILE);
    scan_reduce_kernel<<<(unsigned)nb, SC_THREADS, 0, s>>>(in, n, block_sums);
    scan_block_sums_kernel<<<1, SC_THREADS, 0, s>>>(block_sums, nb);
    scan_downsweep_kernel<<<(unsigned)nb, SC_THREADS, 0, s>>>(in, out, n, block_sums);
    return check_cuda(cudaGetLastError(), "exclusive_scan_u32");
}

static_assert(SC_TILE == SCAN_TILE, "one scan tile size");
int scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *block_sums) {
    return exclusive_scan_u32(s, in, out, n, block_sums);
}

template <typename V, typename I>
__global__ void finalize_kernel(int64_t nnz, const uint64_t *__restrict__ keys,
                                const uint32_t *__restrict__ perm, int minor_bits, int base,
                                const V *__restrict__ val_in, I *__restrict__ idx_out,
                                V *__restrict__ val_out) {
    const uint64_t mask = minor_bits >= 64 ? ~0ull : ((1ull << minor_bits) - 1);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz;
         i += (int64_t)gridDim.x * blockDim.x) {
        idx_out[i] = (I)((int64_t)(keys[i] & mask) + base);
        val_out[i] = ldg(val_in + perm[i]);
    }
}

template <typename I>
__global__ void pointer_kernel(int64_t nnz, const uint64_t *__restrict__ keys, int minor_bits,
                               int64_t major_n, int base, I *__restrict__ ptr_out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nnz;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t prev = i == 0 ? -1 : (int64_t)(keys[i - 1] >> minor_bits);
        int64_t cur = i == nnz ? major_n : (int64_t)(keys[i] >> minor_bits);
        if (cur > major_n) cur = major_n;
        for (int64_t r = prev + 1; r <= cur; ++r) ptr_out[r] = (I)(i + base);
    }
}

struct SortLayout {
    int64_t num_tiles, hist_n;
    size_t bytes;
};
static SortLayout sort_layout(int64_t nnz) {
    SortLayout L;
    L.num_tiles = ceil_div(nnz, RS_TILE);
    L.hist_n = L.num_tiles * RS_BINS;
    Carver cv(nullptr);
    cv.take<uint64_t>(nnz);
    cv.take<uint64_t>(nnz);
    cv.take<uint32_t>(nnz);
    cv.take<uint32_t>(nnz);
    cv.take<uint32_t>(L.hist_n);
    cv.take<uint32_t>(ceil_div(L.hist_n, SC_TILE) + 1);
    L.bytes = align_up(cv.off, 256);
    return L;
}

// The bucket sort applies when the major count, the minor indices and the entry count fit
// its 32-bit fields; the radix sort covers the rest.
static bool bucket_fits(int64_t major_n, int64_t minor_n, int64_t nnz) {
    return major_n + 2 < 0xffffffffLL && minor_n <= 0x100000000LL && nnz < 0xffffffffLL;
}

// Stable LSD radix sort of n (key, payload) pairs over the low total_bits key bits, for
// other translation units: the caller fills the first key and payload buffers of a
// radix_sort_workspace(n)-byte workspace (radix_sort_inputs), and gets back the buffers that
// hold the sorted pairs.
size_t radix_sort_workspace(int64_t n) { return sort_layout(n > 0 ? n : 1).bytes; }
void radix_sort_inputs(void *ws, int64_t n, uint64_t **keys, uint32_t **perm) {
    Carver cv(ws);
    *keys = cv.take<uint64_t>(n);
    cv.take<uint64_t>(n);
    *perm = cv.take<uint32_t>(n);
}
int radix_sort_pairs(cudaStream_t s, void *ws, int64_t n, int total_bits, uint64_t **keys_out, uint32_t **perm_out) {
    const SortLayout L = sort_layout(n > 0 ? n : 1);
    Carver cv(ws);
    uint64_t *ka = cv.take<uint64_t>(n), *kb = cv.take<uint64_t>(n);
    uint32_t *pa = cv.take<uint32_t>(n), *pb = cv.take<uint32_t>(n);
    uint32_t *hist = cv.take<uint32_t>(L.hist_n);
    uint32_t *bsums = cv.take<uint32_t>(ceil_div(L.hist_n, SC_TILE) + 1);
    int rc = GSA_OK;
    for (int shift = 0; n > 0 && shift < total_bits; shift += RS_BITS) {
        const int w = total_bits - shift < RS_BITS ? total_bits - shift : RS_BITS;
        const uint32_t mask = (1u << w) - 1;
        radix_upsweep_kernel<<<(unsigned)L.num_tiles, RS_THREADS, 0, s>>>(ka, n, shift, mask, hist, L.num_tiles);
        rc = exclusive_scan_u32(s, hist, hist, L.hist_n, bsums);
        if (rc) return rc;
        radix_downsweep_kernel<<<(unsigned)L.num_tiles, RS_THREADS, 0, s>>>(ka, pa, kb, pb, n, shift, mask, hist,
                                                                           L.num_tiles);
        rc = check_cuda(cudaGetLastError(), "radix pass");
        if (rc) return rc;
        uint64_t *tk = ka; ka = kb; kb = tk;
        uint32_t *tp = pa; pa = pb; pb = tp;
    }
    *keys_out = ka;
    *perm_out = pa;
    return rc;
}
int radix_bits_for(int64_t count) { return bits_for(count); }

template <typename V, typename I>
size_t coo_to_compressed_workspace_size(int64_t m, int64_t n, int64_t nnz, bool colmajor) {
    if (nnz == 0) return 0;
    const int64_t major_n = colmajor ? n : m, minor_n = colmajor ? m : n;
    if (bucket_fits(major_n, minor_n, nnz)) return bucket::layout(major_n, minor_n, nnz, sizeof(V), SC_TILE).bytes;
    return sort_layout(nnz).bytes;
}

template <typename I>
struct PairSource {
    const I *mj, *mn;
    int base;
    __device__ __forceinline__ int64_t major(int64_t i) const { return (int64_t)__ldg(mj + i) - base; }
    __device__ __forceinline__ void get(int64_t i, int64_t &a, int64_t &b) const {
        a = (int64_t)__ldg(mj + i) - base;
        b = (int64_t)__ldg(mn + i) - base;
    }
};

// Conversion output: pointers from the row starts, minor index from the key, the value
// carried with the key (or gathered by the key's input position).
template <typename V, typename I>
struct CompressedEmit {
    I *ptr_out, *idx_out;
    V *val_out;
    const V *val_in;
    int base;
    int64_t major_n, nnz;
    __device__ __forceinline__ void pointer(int64_t r, uint32_t first) const {
        if (r < major_n) ptr_out[r] = (I)((int64_t)first + base);
        else ptr_out[major_n] = (I)(nnz + base);
    }
    __device__ __forceinline__ void put(uint32_t p, uint64_t, uint64_t key, V v) const {
        idx_out[p] = (I)((int64_t)(key >> 32) + base);
        val_out[p] = v;
    }
    __device__ __forceinline__ void gather(uint32_t p, uint64_t r, uint64_t key) const {
        put(p, r, key, ldg(val_in + (uint32_t)key));
    }
};

static unsigned grid_for(int64_t n, int threads) {
    int64_t b = ceil_div(n, threads);
    if (b > 152 * 32) b = 152 * 32;
    return (unsigned)(b > 0 ? b : 1);
}

template <typename V, typename I>
int launch_coo_to_compressed(cudaStream_t s, bool colmajor, int64_t m, int64_t n, int64_t nnz,
                             const I *rowind, const I *colind, const V *val, int base,
                             I *ptr_out, I *idx_out, V *val_out, void *ws, size_t ws_bytes) {
    const I *major = colmajor ? colind : rowind;
    const I *minor = colmajor ? rowind : colind;
    const int64_t major_n = colmajor ? n : m, minor_n = colmajor ? m : n;
    const int minor_bits = bits_for(minor_n), major_bits = bits_for(major_n);
    if (minor_bits + major_bits > 64)
        return fail(GSA_ERR_UNSUPPORTED, "matrix too large for 64-bit sort keys (%lld x %lld)",
                    (long long)m, (long long)n);
    if (nnz > 0xffffffffLL)
        return fail(GSA_ERR_UNSUPPORTED, "conversion supports at most 2^32-1 stored entries");
    if (nnz == 0) {
        pointer_kernel<I><<<1, 256, 0, s>>>(0, nullptr, minor_bits, major_n, base, ptr_out);
        return check_cuda(cudaGetLastError(), "pointer_kernel");
    }
    if (bucket_fits(major_n, minor_n, nnz)) {
        if (ws_bytes < bucket::layout(major_n, minor_n, nnz, sizeof(V), SC_TILE).bytes)
            return fail(GSA_ERR_INVALID_ARG, "conversion workspace too small");
        PairSource<I> src{major, minor, base};
        CompressedEmit<V, I> emit{ptr_out, idx_out, val_out, val, base, major_n, nnz};
        timer_before(s);
        int rc = bucket::sort(s, major_n, minor_n, nnz, src, val, emit, ws, exclusive_scan_u32, SC_TILE);
        timer_after(s);
        return rc;
    }
    SortLayout L = sort_layout(nnz);
    if (ws_bytes < L.bytes) return fail(GSA_ERR_INVALID_ARG, "conversion workspace too small");
    Carver cv(ws);
    uint64_t *ka = cv.take<uint64_t>(nnz), *kb = cv.take<uint64_t>(nnz);
    uint32_t *pa = cv.take<uint32_t>(nnz), *pb = cv.take<uint32_t>(nnz);
    uint32_t *hist = cv.take<uint32_t>(L.hist_n);
    uint32_t *bsums = cv.take<uint32_t>(ceil_div(L.hist_n, SC_TILE) + 1);

    timer_before(s);
    make_keys_kernel<I><<<grid_for(nnz, 256), 256, 0, s>>>(nnz, major, minor, base, minor_bits, ka, pa);
    int rc = check_cuda(cudaGetLastError(), "make_keys_kernel");
    if (rc) return rc;
    const int total_bits = minor_bits + major_bits;
    for (int shift = 0; shift < total_bits; shift += RS_BITS) {
        int w = total_bits - shift < RS_BITS ? total_bits - shift : RS_BITS;
        uint32_t mask = (1u << w) - 1;
        radix_upsweep_kernel<<<(unsigned)L.num_tiles, RS_THREADS, 0, s>>>(ka, nnz, shift, mask, hist,
                                                                          L.num_tiles);
        rc = exclusive_scan_u32(s, hist, hist, L.hist_n, bsums);
        if (rc) return rc;
        radix_downsweep_kernel<<<(unsigned)L.num_tiles, RS_THREADS, 0, s>>>(
            ka, pa, kb, pb, nnz, shift, mask, hist, L.num_tiles);
        rc = check_cuda(cudaGetLastError(), "radix pass");
        if (rc) return rc;
        uint64_t *tk = ka; ka = kb; kb = tk;
        uint32_t *tp = pa; pa = pb; pb = tp;
    }
    finalize_kernel<V, I><<<grid_for(nnz, 256), 256, 0, s>>>(nnz, ka, pa, minor_bits, base, val,
                                                             idx_out, val_out);
    pointer_kernel<I><<<grid_for(nnz + 1, 256), 256, 0, s>>>(nnz, ka, minor_bits, major_n, base, ptr_out);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "finalize/pointer kernels");
}

// ---------------------------------------------------------------------------
// CSR / CSC -> COO: major index of every stored entry, merge-path tiles.
constexpr int EX_THREADS = 256, EX_IPT = 8, EX_TILE = EX_THREADS * EX_IPT;

template <typename I>
__global__ void __launch_bounds__(EX_THREADS)
expand_major_kernel(int64_t outer_n, int64_t nnz, const I *__restrict__ ptr, int base,
                    const int64_t *__restrict__ coords, I *__restrict__ major_out) {
    __shared__ int s_rowend[EX_TILE];
    __shared__ int s_outer[EX_TILE];
    const int64_t tile = blockIdx.x;
    const int64_t total = outer_n + nnz;
    const int64_t d0 = tile * EX_TILE;
    const int64_t d1 = d0 + EX_TILE < total ? d0 + EX_TILE : total;
    const int64_t rs = coords[tile], re = coords[tile + 1];
    const int64_t js = d0 - rs, je = d1 - re;
    const int tile_rows = (int)(re - rs), tile_nnz = (int)(je - js);
    const int tid = threadIdx.x;
    for (int e = tid; e < tile_rows; e += EX_THREADS)
        s_rowend[e] = (int)((int64_t)__ldg(ptr + rs + 1 + e) - base - js);
    __syncthreads();
    const int items = tile_rows + tile_nnz;
    int d = tid * EX_IPT < items ? tid * EX_IPT : items;
    int lo = d - tile_nnz > 0 ? d - tile_nnz : 0;
    int hi = d < tile_rows ? d : tile_rows;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s_rowend[mid] + mid < d) lo = mid + 1;
        else hi = mid;
    }
    int i = lo, j = d - lo;
#pragma unroll
    for (int step = 0; step < EX_IPT; ++step) {
        if (i < tile_rows && s_rowend[i] <= j) ++i;
        else if (j < tile_nnz) s_outer[j++] = i;
    }
    __syncthreads();
    for (int e = tid; e < tile_nnz; e += EX_THREADS) major_out[js + e] = (I)(rs + s_outer[e] + base);
}

size_t expand_major_workspace_size(int64_t outer_n, int64_t nnz) {
    if (nnz == 0) return 0;
    return align_up((size_t)(ceil_div(outer_n + nnz, EX_TILE) + 1) * sizeof(int64_t), 256);
}

template <typename I>
int launch_expand_major(cudaStream_t s, int64_t outer_n, int64_t nnz, const I *ptr, int base,
                        I *major_out, void *ws, size_t ws_bytes) {
    if (nnz == 0) return GSA_OK;
    if (ws_bytes < expand_major_workspace_size(outer_n, nnz))
        return fail(GSA_ERR_INVALID_ARG, "expansion workspace too small");
    int64_t T = ceil_div(outer_n + nnz, EX_TILE);
    int64_t *coords = (int64_t *)ws;
    int rc = launch_merge_partition<I>(s, ptr, base, outer_n, nnz, EX_TILE, T, coords);
    if (rc) return rc;
    expand_major_kernel<I><<<(unsigned)T, EX_THREADS, 0, s>>>(outer_n, nnz, ptr, base, coords, major_out);
    return check_cuda(cudaGetLastError(), "expand_major_kernel");
}

// ---------------------------------------------------------------------------
// Structure check; flag bits: 1 ptr[0], 2 ptr[end], 4 decreasing ptr, 8 index out of range.
template <typename I>
__global__ void validate_kernel(int64_t outer_n, int64_t inner_n, int64_t nnz, const I *__restrict__ ptr,
                                const I *__restrict__ idx, int base, int *__restrict__ flag) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t0 == 0) {
        if ((int64_t)ptr[0] != base) atomicOr(flag, 1);
        if ((int64_t)ptr[outer_n] != nnz + base) atomicOr(flag, 2);
    }
    for (int64_t o = t0; o < outer_n; o += stride)
        if (ptr[o + 1] < ptr[o]) atomicOr(flag, 4);
    for (int64_t j = t0; j < nnz; j += stride) {
        int64_t v = (int64_t)idx[j] - base;
        if (v < 0 || v >= inner_n) atomicOr(flag, 8);
    }
}

template <typename I>
int launch_validate(cudaStream_t s, int64_t outer_n, int64_t inner_n, int64_t nnz, const I *ptr,
                    const I *idx, int base, int *d_flag) {
    validate_kernel<I><<<grid_for(outer_n > nnz ? outer_n : nnz, 256), 256, 0, s>>>(
        outer_n, inner_n, nnz, ptr, idx, base, d_flag);
    return check_cuda(cudaGetLastError(), "validate_kernel");
}

#define GSA_INST_CONVERT(V, I)                                                                  \
    template int launch_coo_to_compressed<V, I>(cudaStream_t, bool, int64_t, int64_t, int64_t,  \
                                                const I *, const I *, const V *, int, I *, I *, \
                                                V *, void *, size_t);                           \
    template size_t coo_to_compressed_workspace_size<V, I>(int64_t, int64_t, int64_t, bool);
GSA_INST_CONVERT(float, int32_t)
GSA_INST_CONVERT(float, int64_t)
GSA_INST_CONVERT(double, int32_t)
GSA_INST_CONVERT(double, int64_t)
GSA_INST_CONVERT(cf32, int32_t)
GSA_INST_CONVERT(cf32, int64_t)
GSA_INST_CONVERT(cf64, int32_t)
GSA_INST_CONVERT(cf64, int64_t)
GSA_INST_CONVERT(int32_t, int32_t)
GSA_INST_CONVERT(int32_t, int64_t)
GSA_INST_CONVERT(int64_t, int32_t)
GSA_INST_CONVERT(int64_t, int64_t)

template int launch_expand_major<int32_t>(cudaStream_t, int64_t, int64_t, const int32_t *, int,
                                          int32_t *, void *, size_t);
template int launch_expand_major<int64_t>(cudaStream_t, int64_t, int64_t, const int64_t *, int,
                                          int64_t *, void *, size_t);
template int launch_validate<int32_t>(cudaStream_t, int64_t, int64_t, int64_t, const int32_t *,
                                      const int32_t *, int, int *);
template int launch_validate<int64_t>(cudaStream_t, int64_t, int64_t, int64_t, const int64_t *,
                                      const int64_t *, int, int *);

// Row pointers of a row-sorted COO: entry i's predecessor and its own row bound the
// pointer entries it writes (each written once); a decrease or a row outside [0, m)
// clears *sorted instead.
template <typename I>
__global__ void coo_rowptr_kernel(int64_t nnz, const I *__restrict__ rowind, int base, int64_t m,
                                  I *__restrict__ ptr_out, int *sorted) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nnz;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t prev = i == 0 ? -1 : (int64_t)rowind[i - 1] - base;
        const int64_t cur = i == nnz ? m : (int64_t)rowind[i] - base;
        if (cur < prev || cur > m || (i < nnz && cur == m) || prev >= m) {
            atomicExch(sorted, 0);
            continue;
        }
        for (int64_t r = prev + 1; r <= cur; ++r) ptr_out[r] = (I)(i + base);
    }
}

int coo_row_pointers(cudaStream_t s, int itype, int64_t m, int64_t nnz, const void *rowind, int base,
                     void *ptr_out, int *sorted_host) {
    int *flag = nullptr;
    int rc = check_cuda(cudaMallocAsync((void **)&flag, sizeof(int), s), "coo plan: flag");
    if (rc) return rc;
    const int one = 1;
    rc = check_cuda(cudaMemcpyAsync(flag, &one, sizeof(int), cudaMemcpyHostToDevice, s), "coo plan: flag");
    if (!rc) {
        int64_t blocks = ceil_div(nnz + 1, 256);
        if (blocks > 152 * 64) blocks = 152 * 64;
        if (itype == GSA_IDX32)
            coo_rowptr_kernel<int32_t><<<(unsigned)blocks, 256, 0, s>>>(nnz, (const int32_t *)rowind, base, m,
                                                                         (int32_t *)ptr_out, flag);
        else
            coo_rowptr_kernel<int64_t><<<(unsigned)blocks, 256, 0, s>>>(nnz, (const int64_t *)rowind, base, m,
                                                                         (int64_t *)ptr_out, flag);
        rc = check_cuda(cudaGetLastError(), "coo_rowptr_kernel");
    }
    if (!rc) rc = check_cuda(cudaMemcpyAsync(sorted_host, flag, sizeof(int), cudaMemcpyDeviceToHost, s),
                             "coo plan: flag");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "coo plan: sync");
    cudaFreeAsync(flag, s);
    return rc;
}

// ---------------------------------------------------------------------------
// COO sums: A + B, A + λI and duplicate compaction (src/matrix_coo/matrix_coo.jl:300-385,
// 387-458 and the transposed pairs at :460-575; kernels kernel_mark_unique_coo! and
// kernel_compact_coo! at src/matrix_coo/matrix_coo_kernels.jl:257-311, followed there by
// dropzeros).  The reference concatenates the sources, sorts column-major keys, marks run
// starts, cumsums the marks, sums every run in its sorted order into a new COO and then
// drops the zero sums with a second compaction.  Here the sources are read where they lie
// (no concatenation): entry p < nnz_a is A's (indices swapped when A is transposed, value
// conjugated when adjoint), then B's, then the n_diag diagonal entries of λI.  One stable
// radix sort of 64-bit keys (col << row_bits | row); then one kernel sums each run where it
// starts (left to right in sorted order, which is storage order within a source) and flags
// the nonzero sums; one scan gives the positions and the count.  The copy phase writes the
// flagged runs.  Zero sums never reach the output, so no second compaction is needed.

template <typename I>
__global__ void sum_keys_kernel(SumSources src, int64_t total, int base, int row_bits, uint64_t *__restrict__ keys,
                                uint32_t *__restrict__ perm) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r, c;
        if (i < src.nnz[0] + src.nnz[1]) {
            const int w = i < src.nnz[0] ? 0 : 1;
            const int64_t j = w ? i - src.nnz[0] : i;
            const int64_t ri = (int64_t)ld_stream((const I *)src.row[w] + j) - base;
            const int64_t ci = (int64_t)ld_stream((const I *)src.col[w] + j) - base;
            r = src.trans[w] ? ci : ri;
            c = src.trans[w] ? ri : ci;
        } else {
            r = c = i - src.nnz[0] - src.nnz[1];
        }
        keys[i] = row_bits >= 64 ? (uint64_t)r : (((uint64_t)c << row_bits) | (uint64_t)r);
        perm[i] = (uint32_t)i;
    }
}

template <typename V> __device__ __forceinline__ V negate_if(V a, bool c) {  // integers wrap, as in Julia
    using U = typename std::make_unsigned<V>::type;
    return c ? (V)(U(0) - (U)a) : a;
}
template <> __device__ __forceinline__ float negate_if(float a, bool c) { return flip_sign_if(a, c); }
template <> __device__ __forceinline__ double negate_if(double a, bool c) { return flip_sign_if(a, c); }
template <> __device__ __forceinline__ cf32 negate_if(cf32 a, bool c) {
    return cf32{flip_sign_if(a.re, c), flip_sign_if(a.im, c)};
}
template <> __device__ __forceinline__ cf64 negate_if(cf64 a, bool c) {
    return cf64{flip_sign_if(a.re, c), flip_sign_if(a.im, c)};
}

template <typename V>
__device__ __forceinline__ V sum_source_value(const SumSources &src, uint32_t p, V lambda) {
    if (p >= src.nnz[0] + src.nnz[1]) return lambda;
    const int w = p < src.nnz[0] ? 0 : 1;
    const V v = ldg((const V *)src.val[w] + (w ? p - src.nnz[0] : p));
    return negate_if(conj_if(v, src.conj[w] != 0), src.neg[w] != 0);
}

// flags[i] = 1 where sorted entry i starts a run whose sum is nonzero; the sum goes to sums[i].
template <typename V>
__global__ void run_sum_kernel(SumSources src, int64_t total, const uint64_t *__restrict__ keys,
                               const uint32_t *__restrict__ perm, V lambda, V *__restrict__ sums,
                               uint32_t *__restrict__ flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= total; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        if (i < total) {
            const uint64_t k = keys[i];
            if (i == 0 || keys[i - 1] != k) {
                V acc = sum_source_value<V>(src, perm[i], lambda);
                for (int64_t j = i + 1; j < total && keys[j] == k; ++j)
                    acc = add(acc, sum_source_value<V>(src, perm[j], lambda));
                sums[i] = acc;
                f = is_zero(acc) ? 0u : 1u;
            }
        }
        flags[i] = f;
    }
}

template <typename V, typename I>
__global__ void run_write_kernel(int64_t total, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ pos,
                                 const V *__restrict__ sums, int row_bits, int base, I *__restrict__ row_out,
                                 I *__restrict__ col_out, V *__restrict__ val_out) {
    const uint64_t mask = row_bits >= 64 ? ~0ull : ((1ull << row_bits) - 1);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = pos[i];
        if (pos[i + 1] == p) continue;  // not a run start, or a zero sum
        const uint64_t k = keys[i];
        row_out[p] = (I)((int64_t)(k & mask) + base);
        col_out[p] = (I)((int64_t)(row_bits >= 64 ? 0 : k >> row_bits) + base);
        val_out[p] = sums[i];
    }
}

// Column-major order: buckets are columns, the minor index is the row.
template <typename I>
struct SumSource {
    SumSources s;
    int base;
    __device__ __forceinline__ void get(int64_t i, int64_t &col, int64_t &row) const {
        if (i < s.nnz[0] + s.nnz[1]) {
            const int w = i < s.nnz[0] ? 0 : 1;
            const int64_t j = w ? i - s.nnz[0] : i;
            const int64_t ri = (int64_t)__ldg((const I *)s.row[w] + j) - base;
            const int64_t ci = (int64_t)__ldg((const I *)s.col[w] + j) - base;
            row = s.trans[w] ? ci : ri;
            col = s.trans[w] ? ri : ci;
        } else {
            row = col = i - s.nnz[0] - s.nnz[1];
        }
    }
    __device__ __forceinline__ int64_t major(int64_t i) const {
        int64_t c, r;
        get(i, c, r);
        return c;
    }
};

// Sorted (col << 32 | row) keys and input positions, for the run kernels.
struct KeyEmit {
    uint64_t *keys;
    uint32_t *perm;
    __device__ __forceinline__ void pointer(int64_t, uint32_t) const {}
    __device__ __forceinline__ void gather(uint32_t p, uint64_t col, uint64_t key) const {
        keys[p] = (col << 32) | (key >> 32);
        perm[p] = (uint32_t)key;
    }
};

struct SumLayout {
    bool bucket;
    SortLayout sort;
    size_t keys, perm, flags, pos, bsums, sums, bytes;
};
static SumLayout sum_layout(int64_t m, int64_t n, int64_t total, size_t vsize) {
    SumLayout L;
    L.bucket = bucket_fits(n, m, total);
    Carver cv(nullptr);
    if (L.bucket) {
        cv.reserve<unsigned char>(bucket::layout(n, m, total, 0, SC_TILE).bytes);
        L.keys = cv.reserve<uint64_t>(total);
        L.perm = cv.reserve<uint32_t>(total);
    } else {
        L.sort = sort_layout(total);
        cv.take<unsigned char>(L.sort.bytes);
        // the radix sort leaves its result in the first or second key buffer, by the parity
        // of its pass count
        const int passes = (bits_for(m) + bits_for(n) + RS_BITS - 1) / RS_BITS;
        Carver sc(nullptr);  // the buffers in the order the sort takes them
        sc.reserve<uint64_t>(total);
        const size_t kb = sc.reserve<uint64_t>(total);
        const size_t pa = sc.reserve<uint32_t>(total);
        const size_t pb = sc.reserve<uint32_t>(total);
        L.keys = passes % 2 ? kb : 0;
        L.perm = passes % 2 ? pb : pa;
    }
    L.flags = cv.reserve<uint32_t>(total + 1);
    L.pos = cv.reserve<uint32_t>(total + 1);
    L.bsums = cv.reserve<uint32_t>(ceil_div(total + 1, SC_TILE) + 1);
    L.sums = cv.reserve<unsigned char>((size_t)total * vsize);
    L.bytes = align_up(cv.off, 256);
    return L;
}

size_t coo_sum_workspace_size(size_t vsize, int64_t m, int64_t n, int64_t total) {
    return total <= 0 ? 256 : sum_layout(m, n, total, vsize).bytes;
}

template <typename V, typename I>
int launch_coo_sum_count(cudaStream_t s, int64_t m, int64_t n, const SumSources &src, const V *lambda, int base,
                         void *ws, size_t ws_bytes, int64_t *kept) {
    const int64_t total = src.nnz[0] + src.nnz[1] + src.n_diag;
    if (total + 1 > 0xffffffffLL) return fail(GSA_ERR_UNSUPPORTED, "at most 2^32 - 2 entries in a sum");
    const int row_bits = bits_for(m), col_bits = bits_for(n);
    if (row_bits + col_bits > 64)
        return fail(GSA_ERR_UNSUPPORTED, "matrix too large for 64-bit sort keys (%lld x %lld)", (long long)m,
                    (long long)n);
    if (ws_bytes < coo_sum_workspace_size(sizeof(V), m, n, total))
        return fail(GSA_ERR_INVALID_ARG, "workspace too small");
    if (total == 0) {
        *kept = 0;
        return GSA_OK;
    }
    const SumLayout L = sum_layout(m, n, total, sizeof(V));
    char *w = (char *)ws;
    uint64_t *keys = (uint64_t *)(w + L.keys);
    uint32_t *perm = (uint32_t *)(w + L.perm);
    uint32_t *flags = (uint32_t *)(w + L.flags), *pos = (uint32_t *)(w + L.pos);
    uint32_t *bs2 = (uint32_t *)(w + L.bsums);
    V *sums = (V *)(w + L.sums);
    int rc = GSA_OK;
    timer_before(s);
    if (L.bucket) {
        SumSource<I> bs{src, base};
        rc = bucket::sort(s, n, m, total, bs, (const bucket::NoValue *)nullptr, KeyEmit{keys, perm}, ws,
                          exclusive_scan_u32, SC_TILE);
    } else {
        Carver cv(ws);
        uint64_t *ka = cv.take<uint64_t>(total), *kb = cv.take<uint64_t>(total);
        uint32_t *pa = cv.take<uint32_t>(total), *pb = cv.take<uint32_t>(total);
        uint32_t *hist = cv.take<uint32_t>(L.sort.hist_n);
        uint32_t *bsums = cv.take<uint32_t>(ceil_div(L.sort.hist_n, SC_TILE) + 1);
        sum_keys_kernel<I><<<grid_for(total, 256), 256, 0, s>>>(src, total, base, row_bits, ka, pa);
        rc = check_cuda(cudaGetLastError(), "sum_keys_kernel");
        const int total_bits = row_bits + col_bits;
        for (int shift = 0; !rc && shift < total_bits; shift += RS_BITS) {
            const int wb = total_bits - shift < RS_BITS ? total_bits - shift : RS_BITS;
            const uint32_t mask = (1u << wb) - 1;
            radix_upsweep_kernel<<<(unsigned)L.sort.num_tiles, RS_THREADS, 0, s>>>(ka, total, shift, mask, hist,
                                                                                   L.sort.num_tiles);
            rc = exclusive_scan_u32(s, hist, hist, L.sort.hist_n, bsums);
            if (rc) break;
            radix_downsweep_kernel<<<(unsigned)L.sort.num_tiles, RS_THREADS, 0, s>>>(ka, pa, kb, pb, total, shift,
                                                                                     mask, hist, L.sort.num_tiles);
            rc = check_cuda(cudaGetLastError(), "radix pass");
            uint64_t *tk = ka; ka = kb; kb = tk;
            uint32_t *tp = pa; pa = pb; pb = tp;
        }
        if (!rc && (ka != keys || pa != perm)) rc = fail(GSA_ERR_CUDA, "coo sum: sorted keys not where expected");
    }
    if (!rc) {
        const V lam = lambda ? *lambda : V{};
        run_sum_kernel<V><<<grid_for(total + 1, 256), 256, 0, s>>>(src, total, keys, perm, lam, sums, flags);
        rc = check_cuda(cudaGetLastError(), "run_sum_kernel");
    }
    if (!rc) rc = exclusive_scan_u32(s, flags, pos, total + 1, bs2);
    timer_after(s);
    uint32_t u = 0;
    if (!rc) rc = check_cuda(cudaMemcpyAsync(&u, pos + total, sizeof(u), cudaMemcpyDeviceToHost, s), "coo sum: count");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "coo sum: sync");
    if (!rc) *kept = (int64_t)u;
    return rc;
}

template <typename V, typename I>
int launch_coo_sum_copy(cudaStream_t s, int64_t m, int64_t n, int64_t total, int base, const void *ws, I *row_out,
                        I *col_out, V *val_out) {
    if (total <= 0) return GSA_OK;
    const SumLayout L = sum_layout(m, n, total, sizeof(V));
    const char *w = (const char *)ws;
    const uint64_t *keys = (const uint64_t *)(w + L.keys);
    const uint32_t *pos = (const uint32_t *)(w + L.pos);
    const V *sums = (const V *)(w + L.sums);
    timer_before(s);
    run_write_kernel<V, I><<<grid_for(total, 256), 256, 0, s>>>(total, keys, pos, sums, L.bucket ? 32 : bits_for(m),
                                                               base, row_out, col_out, val_out);
    timer_after(s);
    return check_cuda(cudaGetLastError(), "run_write_kernel");
}

#define GSA_INST_COOSUM(V, I)                                                                                  \
    template int launch_coo_sum_count<V, I>(cudaStream_t, int64_t, int64_t, const SumSources &, const V *, int, \
                                            void *, size_t, int64_t *);                                       \
    template int launch_coo_sum_copy<V, I>(cudaStream_t, int64_t, int64_t, int64_t, int, const void *, I *, I *, \
                                           V *);
GSA_INST_COOSUM(float, int32_t) GSA_INST_COOSUM(float, int64_t) GSA_INST_COOSUM(double, int32_t)
GSA_INST_COOSUM(double, int64_t) GSA_INST_COOSUM(cf32, int32_t) GSA_INST_COOSUM(cf32, int64_t)
GSA_INST_COOSUM(cf64, int32_t) GSA_INST_COOSUM(cf64, int64_t) GSA_INST_COOSUM(int32_t, int32_t)
GSA_INST_COOSUM(int32_t, int64_t) GSA_INST_COOSUM(int64_t, int32_t) GSA_INST_COOSUM(int64_t, int64_t)

// ---------------------------------------------------------------------------
// dropzeros (src/matrix_csr/matrix_csr.jl:649-745 with kernel_count_nonzeros_csr! /
// kernel_dropzeros_csr!, src/matrix_csr/matrix_csr_kernels.jl:409-443; the CSC and COO
// counterparts): the stored entries that are not zero, in storage order.  Here one flag
// per entry, one exclusive scan (the kept entries' new positions, and at [nnz] their
// count), a scatter of the kept entries, and the new pointer of outer entry r is the
// position of its first entry -- no per-row loop, so long rows cost nothing extra.

template <typename V>
__global__ void nonzero_flags_kernel(int64_t nnz, const V *__restrict__ val, uint32_t *__restrict__ flags) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nnz; i += (int64_t)gridDim.x * blockDim.x)
        flags[i] = i < nnz && !is_zero(ldg(val + i)) ? 1u : 0u;
}

template <typename V, typename I>
__global__ void drop_scatter_kernel(int64_t nnz, const uint32_t *__restrict__ pos, const I *__restrict__ i0,
                                    const I *__restrict__ i1, const V *__restrict__ val, I *__restrict__ o0,
                                    I *__restrict__ o1, V *__restrict__ ov) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t p = pos[i];
        if (pos[i + 1] == p) continue;  // a zero
        if (i0) o0[p] = i0[i];
        o1[p] = i1[i];
        ov[p] = val[i];
    }
}

template <typename I>
__global__ void drop_pointer_kernel(int64_t outer_n, int64_t nnz, const I *__restrict__ ptr, int base,
                                    const uint32_t *__restrict__ pos, I *__restrict__ ptr_out) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= outer_n; r += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = (int64_t)ptr[r] - base;
        j = j < 0 ? 0 : (j > nnz ? nnz : j);
        ptr_out[r] = (I)((int64_t)pos[j] + base);
    }
}

size_t dropzeros_workspace_size(int64_t nnz) {
    Carver cv(nullptr);
    cv.take<uint32_t>(nnz + 1);
    cv.take<uint32_t>(nnz + 1);
    cv.take<uint32_t>(ceil_div(nnz + 1, SC_TILE) + 1);
    return align_up(cv.off, 256);
}

template <typename V>
int launch_dropzeros_count(cudaStream_t s, int64_t nnz, const V *val, void *ws, size_t ws_bytes, int64_t *kept) {
    if (nnz + 1 > 0xffffffffLL) return fail(GSA_ERR_UNSUPPORTED, "dropzeros: more than 2^32 - 1 entries");
    if (ws_bytes < dropzeros_workspace_size(nnz)) return fail(GSA_ERR_INVALID_ARG, "dropzeros workspace too small");
    Carver cv(ws);
    uint32_t *flags = cv.take<uint32_t>(nnz + 1);
    uint32_t *pos = cv.take<uint32_t>(nnz + 1);
    uint32_t *bsums = cv.take<uint32_t>(ceil_div(nnz + 1, SC_TILE) + 1);
    int64_t blocks = ceil_div(nnz + 1, 256);
    if (blocks > 152 * 64) blocks = 152 * 64;
    nonzero_flags_kernel<V><<<(unsigned)blocks, 256, 0, s>>>(nnz, val, flags);
    int rc = check_cuda(cudaGetLastError(), "nonzero_flags_kernel");
    if (!rc) rc = exclusive_scan_u32(s, flags, pos, nnz + 1, bsums);
    uint32_t total = 0;
    if (!rc) rc = check_cuda(cudaMemcpyAsync(&total, pos + nnz, sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                             "dropzeros: count");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s), "dropzeros: sync");
    if (!rc) *kept = (int64_t)total;
    return rc;
}

template <typename V, typename I>
int launch_dropzeros_copy(cudaStream_t s, int fmt, int64_t outer_n, int64_t nnz, const I *p0, const I *p1,
                          const V *val, int base, const void *ws, I *o0, I *o1, V *ov) {
    Carver cv(const_cast<void *>(ws));
    cv.take<uint32_t>(nnz + 1);
    const uint32_t *pos = cv.take<uint32_t>(nnz + 1);
    int64_t blocks = ceil_div(nnz > outer_n ? nnz : outer_n + 1, 256);
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (blocks < 1) blocks = 1;
    if (nnz > 0)
        drop_scatter_kernel<V, I><<<(unsigned)blocks, 256, 0, s>>>(nnz, pos, fmt == 2 ? p0 : nullptr, p1, val,
                                                                  fmt == 2 ? o0 : nullptr, o1, ov);
    if (fmt != 2)
        drop_pointer_kernel<I><<<(unsigned)blocks, 256, 0, s>>>(outer_n, nnz, p0, base, pos, o0);
    return check_cuda(cudaGetLastError(), "dropzeros copy");
}

#define GSA_INST_DROP_V(V) template int launch_dropzeros_count<V>(cudaStream_t, int64_t, const V *, void *, size_t, int64_t *);
#define GSA_INST_DROP(V, I)                                                                          \
    template int launch_dropzeros_copy<V, I>(cudaStream_t, int, int64_t, int64_t, const I *, const I *, \
                                             const V *, int, const void *, I *, I *, V *);
GSA_INST_DROP_V(float) GSA_INST_DROP_V(double) GSA_INST_DROP_V(cf32) GSA_INST_DROP_V(cf64)
GSA_INST_DROP_V(int32_t) GSA_INST_DROP_V(int64_t)
GSA_INST_DROP(float, int32_t) GSA_INST_DROP(float, int64_t) GSA_INST_DROP(double, int32_t)
GSA_INST_DROP(double, int64_t) GSA_INST_DROP(cf32, int32_t) GSA_INST_DROP(cf32, int64_t)
GSA_INST_DROP(cf64, int32_t) GSA_INST_DROP(cf64, int64_t) GSA_INST_DROP(int32_t, int32_t)
GSA_INST_DROP(int32_t, int64_t) GSA_INST_DROP(int64_t, int32_t) GSA_INST_DROP(int64_t, int64_t)

}  // namespace gsa
