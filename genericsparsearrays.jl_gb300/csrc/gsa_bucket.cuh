// Stable sort of (major, minor) pairs by bucketing on the major index.
//
// The conversions (COO -> CSR / CSC) and the COO sums order their entries by (major, minor)
// with ties kept in input order.  Instead of an LSD radix sort over all key bits (six passes
// of 8-bit digits for a 4M x 4M matrix), the entries are bucketed by their major index and
// each bucket (one row of the result) is sorted on its own by (minor, input position), which
// gives the order of a stable sort.  Every entry carries the key minor << 32 | position.
//
// Two levels, so that no pass writes single entries to random addresses (a random 8-byte
// store costs a whole DRAM sector, and more):
//   A. coarse_count_kernel: entries per coarse bucket (2^cs consecutive rows, at most 4096
//      rows and 8192 buckets), histograms in shared memory; one scan of the bucket counts.
//   B. coarse_place_kernel: a CTA takes a tile of 2048 entries, ranks them per coarse bucket
//      in shared memory and reserves one contiguous run per bucket with one global atomic,
//      so the tile's writes land in runs that L2 merges into whole sectors.  Each entry is one
//      record: the key row-in-bucket << (mb + pb) | minor << pb | position (sorting a row by it
//      is sorting by (minor, position)) and the value (conversions), one 16- or 32-byte store.
//   C. fine_kernel: a CTA per coarse bucket counts its rows in shared memory, scans them --
//      the row pointers of the result -- and places the bucket's entries in row order into
//      shared memory (96 KB of staging; cs is chosen so that an average bucket fills at most
//      half of it).  Rows of up to 16 entries are sorted there by a thread in registers (rank
//      counting), rows of up to 256 by a warp, and emitted; longer rows go to cta_kernel
//      (rank counting up to 1024 entries, else a bitonic sort of 16384-entry chunks in shared
//      memory, merged pairwise; values then gathered by input position).  A bucket larger than the staging is placed in global
//      memory instead, with its rows of more than 16 entries listed for warp_kernel and
//      cta_kernel.  Where rows average at most 8 entries, fine_stage_kernel runs this pass
//      instead: one CTA per SM, the next bucket's records copied into shared memory while the
//      current one is sorted, the bucket's output written with coalesced stores.
// Matrices with more than 8191 x 4096 rows take the one-level form (count, place, and
// small_kernel per row), whose stores are random.
//
// A source gives, for entry i, its 0-based major index (`major(i)`) and both indices
// (`get(i, major, minor)`); an emitter receives each row's first position (`pointer(r,
// first)`, r = 0..major_n) and every entry's sorted position with its row, key and value
// (`put(p, r, key, value)`, or `gather(p, r, key)` where the value is not carried).
//
// Requirements: major_n < 2^32 - 2, minor indices < 2^32 and fewer than 2^32 - 1 entries.
// Entries whose major index is outside [0, major_n) go to one extra row after the last (and
// one extra coarse bucket), so that no index leaves its array.
#pragma once

#include <type_traits>

#include "gsa_internal.cuh"

namespace gsa {
namespace bucket {

constexpr int SMALL = 16;          // a thread sorts rows of up to 16 entries in registers
constexpr int WARP_MAX = 256;      // a warp sorts rows of up to 256 entries
constexpr int CTA_THREADS = 1024;
constexpr int CTA_TILE = 16384;    // a CTA sorts 16384 entries in shared memory at once (128 KB)
constexpr int RANK_MAX = 1024;     // a CTA ranks rows of up to 1024 entries by counting
constexpr int WARP_CTA_THREADS = 256;
constexpr int MERGE_ITEMS = 8;
constexpr int ROWS_MAX = 4096;     // rows per coarse bucket
constexpr int COARSE_MAX = 8192;   // coarse buckets, the invalid-row bucket included
constexpr int PB_THREADS = 256, PB_ITEMS = 8;
constexpr int PC_THREADS = 512;
constexpr int STAGE_BYTES = 96 * 1024;  // fine_kernel's shared staging of one coarse bucket

struct NoValue {};  // the COO sums carry no values (they sum by input position)

template <class VT> __host__ __device__ constexpr size_t carried_size() {
    return std::is_same<VT, NoValue>::value ? 0 : sizeof(VT);
}
// Entries of a coarse bucket that fine_kernel stages in shared memory (key + value each).
template <class VT> __host__ __device__ constexpr int stage_entries() { return (int)(STAGE_BYTES / (8 + carried_size<VT>())); }

struct Coarse {
    bool ok;
    int cs;       // rows per coarse bucket = 2^cs
    int64_t nb;   // coarse buckets, the last one for invalid rows
    int mb, pb;   // bits of the minor index and of the entry position in the packed keys
};
inline int nbits(int64_t count) {  // bits that values 0 .. count - 1 need
    int b = 0;
    while (b < 63 && ((int64_t)1 << b) < count) ++b;
    return b;
}
// The fewest rows per bucket that keep the bucket count in bounds, raised while a bucket of
// average rows still fills at most half the shared staging.  The two-level form packs the
// row inside the bucket, the minor index and the position into one 64-bit key, so the three
// must fit.
inline Coarse coarse_plan(int64_t major_n, int64_t minor_n, int64_t nnz, int stage) {
    Coarse c{false, 0, 0, 0, 0};
    int cs = 0;
    while (cs < 40 && ((major_n + ((int64_t)1 << cs) - 1) >> cs) + 1 > COARSE_MAX) ++cs;
    const double avg = major_n > 0 ? (double)nnz / (double)major_n : 0.0;
    while (cs < 12 && (double)((int64_t)2 << cs) * avg <= 0.5 * stage) ++cs;
    if (((int64_t)1 << cs) > ROWS_MAX) return c;
    c.mb = nbits(minor_n);
    c.pb = nbits(nnz);
    if (c.mb + c.pb + cs > 64) return c;
    c.ok = true;
    c.cs = cs;
    c.nb = ((major_n + ((int64_t)1 << cs) - 1) >> cs) + 1;
    return c;
}

// Pass B's record: the packed key and the carried value, stored together (one 16- or 32-byte
// store per entry).
template <class VT, bool HAS = !std::is_same<VT, NoValue>::value> struct Rec;
template <class VT> struct alignas(16) Rec<VT, true> {
    uint64_t key;
    VT val;
};
template <class VT> struct Rec<VT, false> {
    uint64_t key;
};
constexpr size_t rec_size(size_t vsize) { return vsize == 0 ? 8 : (vsize <= 8 ? 16 : 32); }

// Stores a record with every byte written, the alignment padding as zeros (4-byte values
// leave 4 bytes, 16-byte values 8 bytes): a sector left partly unwritten makes the L2 read it
// from DRAM before writing it back, which doubled pass B's reads for ComplexF64.
template <class VT> __device__ __forceinline__ void store_rec(Rec<VT> *p, uint64_t key, const VT &v) {
    static_assert(sizeof(VT) == 4 || sizeof(VT) == 8 || sizeof(VT) == 16, "record values of 4, 8 or 16 bytes");
    if constexpr (sizeof(VT) == 16) {
        ulonglong2 head, tail;
        head.x = key;
        head.y = 0;
        memcpy(&tail, &v, 16);
        reinterpret_cast<ulonglong2 *>(p)[0] = head;
        reinterpret_cast<ulonglong2 *>(p)[1] = tail;
    } else {
        ulonglong2 w;
        w.x = key;
        w.y = 0;
        memcpy(&w.y, &v, sizeof(VT));
        *reinterpret_cast<ulonglong2 *>(p) = w;
    }
}
__device__ __forceinline__ void store_rec(Rec<NoValue> *p, uint64_t key, NoValue) { p->key = key; }

__host__ __device__ __forceinline__ uint64_t shl64(uint64_t x, int n) { return n >= 64 ? 0 : x << n; }
__host__ __device__ __forceinline__ uint64_t shr64(uint64_t x, int n) { return n >= 64 ? 0 : x >> n; }
__host__ __device__ __forceinline__ uint64_t low_mask(int n) { return n >= 64 ? ~0ull : (1ull << n) - 1; }

// row << (mb + pb) | minor << pb | position  ->  minor << 32 | position
__device__ __forceinline__ uint64_t canonical_key(uint64_t k, int mb, int pb) {
    return (((k >> pb) & low_mask(mb)) << 32) | (k & low_mask(pb));
}

// An emitter seen through packed keys: keys are turned back into minor << 32 | position.
template <class Emit> struct PackedEmit {
    Emit e;
    int mb, pb;
    __device__ __forceinline__ void pointer(int64_t r, uint32_t first) const { e.pointer(r, first); }
    template <class V> __device__ __forceinline__ void put(uint32_t p, uint64_t r, uint64_t key, V v) const {
        e.put(p, r, canonical_key(key, mb, pb), v);
    }
    __device__ __forceinline__ void gather(uint32_t p, uint64_t r, uint64_t key) const {
        e.gather(p, r, canonical_key(key, mb, pb));
    }
};

struct Layout {
    Coarse co;
    int64_t ncnt;
    size_t cnt, cstart, start, bsums, key1, rec1, key2, val2, list, counters, bytes;
};

// vsize: bytes of a carried value (0: none)
inline Layout layout(int64_t major_n, int64_t minor_n, int64_t nnz, size_t vsize, size_t sc_tile) {
    Layout L;
    L.co = coarse_plan(major_n, minor_n, nnz, (int)(STAGE_BYTES / (8 + vsize)));
    const int64_t n = nnz > 0 ? nnz : 1;
    L.ncnt = (L.co.ok ? L.co.nb : major_n) + 2;
    const int64_t nscan = L.ncnt > major_n + 2 ? L.ncnt : major_n + 2;
    Carver cv(nullptr);
    L.cnt = cv.reserve<uint32_t>(L.ncnt);
    L.cstart = cv.reserve<uint32_t>(L.ncnt);
    L.start = cv.reserve<uint32_t>(major_n + 2);
    L.bsums = cv.reserve<uint32_t>(ceil_div(nscan, (int64_t)sc_tile) + 1);
    L.key1 = cv.reserve<uint64_t>(n);
    L.key2 = cv.reserve<uint64_t>(n);
    L.rec1 = L.co.ok ? cv.reserve<unsigned char>((size_t)n * rec_size(vsize)) : 0;
    L.val2 = L.co.ok && vsize ? cv.reserve<unsigned char>((size_t)n * vsize) : 0;
    L.list = cv.reserve<uint32_t>(major_n + 1);
    L.counters = cv.reserve<uint32_t>(4);
    L.bytes = align_up(cv.off, 256);
    return L;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return lt;
}

template <class Emit, class VT>
__device__ __forceinline__ void emit_one(const Emit &e, uint32_t p, uint64_t r, uint64_t key, const VT *vals,
                                         uint32_t at) {
    if constexpr (std::is_same<VT, NoValue>::value) {
        e.gather(p, r, key);
    } else {
        if (vals) e.put(p, r, key, vals[at]);
        else e.gather(p, r, key);
    }
}

// Rank-counting sort of one row of up to N keys in registers (keys / vals point at the
// row's first entry; the value of the key at slot j moves with it), emitted from position
// `out`.  keys / vals may have been written earlier in the same kernel: plain loads.
template <class Emit, class VT, int N>
__device__ __forceinline__ void sort_registers(const uint64_t *keys, const VT *vals, uint32_t out, uint32_t len,
                                               uint64_t r, const Emit &emit) {
    uint64_t k[N];
#pragma unroll
    for (int j = 0; j < N; ++j) k[j] = (uint32_t)j < len ? keys[j] : ~0ull;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if ((uint32_t)j >= len) break;
        uint32_t rank = 0;
#pragma unroll
        for (int q = 0; q < N; ++q) rank += k[q] < k[j] ? 1u : 0u;
        emit_one(emit, out + rank, r, k[j], vals, (uint32_t)j);
    }
}

template <class Emit, class VT>
__device__ __forceinline__ void sort_short_row(const uint64_t *keys, const VT *vals, uint32_t out, uint32_t len,
                                               uint64_t r, const Emit &emit) {
    if (len <= 4) sort_registers<Emit, VT, 4>(keys, vals, out, len, r, emit);
    else if (len <= 8) sort_registers<Emit, VT, 8>(keys, vals, out, len, r, emit);
    else if (len <= SMALL) sort_registers<Emit, VT, SMALL>(keys, vals, out, len, r, emit);
}

// Rows longer than SMALL go to the lists: warp-sized from the front, CTA-sized from the
// back (one atomic per warp and list).  All 32 lanes call this.
__device__ __forceinline__ void list_long_rows(bool valid, uint32_t len, uint32_t r, int64_t major_n,
                                               uint32_t *list, uint32_t *counters) {
    const bool to_warp = valid && len > SMALL && len <= WARP_MAX;
    const bool to_cta = valid && len > WARP_MAX;
    const unsigned mw = __ballot_sync(0xffffffffu, to_warp), mc = __ballot_sync(0xffffffffu, to_cta);
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    uint32_t bw = 0, bc = 0;
    if (lane == 0 && mw) bw = atomicAdd(&counters[0], (uint32_t)__popc(mw));
    if (lane == 0 && mc) bc = atomicAdd(&counters[1], (uint32_t)__popc(mc));
    bw = __shfl_sync(0xffffffffu, bw, 0);
    bc = __shfl_sync(0xffffffffu, bc, 0);
    if (to_warp) list[bw + __popc(mw & lt)] = r;
    if (to_cta) list[major_n - (bc + __popc(mc & lt))] = r;
}

// ---- two-level form --------------------------------------------------------

template <class Src>
__global__ void __launch_bounds__(PB_THREADS)
coarse_count_kernel(Src src, int64_t nnz, int64_t major_n, int cs, int64_t nb, uint32_t *__restrict__ cnt) {
    __shared__ uint32_t h[COARSE_MAX];
    for (int64_t d = threadIdx.x; d < nb; d += blockDim.x) h[d] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // eight loads in flight per thread before their shared-memory atomics
    for (; i + 7 * stride < nnz; i += 8 * stride) {
        int64_t mj[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) mj[u] = src.major(i + u * stride);
#pragma unroll
        for (int u = 0; u < 8; ++u) atomicAdd(&h[(uint64_t)mj[u] < (uint64_t)major_n ? mj[u] >> cs : nb - 1], 1u);
    }
    for (; i < nnz; i += stride) {
        const int64_t mj = src.major(i);
        atomicAdd(&h[(uint64_t)mj < (uint64_t)major_n ? mj >> cs : nb - 1], 1u);
    }
    __syncthreads();
    for (int64_t d = threadIdx.x; d < nb; d += blockDim.x)
        if (h[d]) atomicAdd(&cnt[d], h[d]);
}

// Resident CTAs of the placement: 4 (64 registers, half the SM's warps) measured 631 us for
// the permuted Laplacian F64/I64 conversion against 666 us with 3 (80 registers), 664 with 5 and
// 683 with 6 (both spilling); the power-law ComplexF64 conversion is the same within noise.
#ifndef GSA_PB_MIN_BLOCKS
#define GSA_PB_MIN_BLOCKS 4
#endif
template <class Src, class VT>
__global__ void __launch_bounds__(PB_THREADS, GSA_PB_MIN_BLOCKS)
coarse_place_kernel(Src src, const VT *__restrict__ vals_in, int64_t nnz, int64_t major_n, Coarse co,
                    uint32_t *__restrict__ cfill, Rec<VT> *__restrict__ rec1) {
    const int cs = co.cs;
    const int64_t nb = co.nb;
    // per bucket: the tile's count, then (in place) the first slot of the tile's run
    __shared__ uint32_t s_run[COARSE_MAX];
    constexpr bool HAS_VAL = !std::is_same<VT, NoValue>::value;
    constexpr int64_t TILE = (int64_t)PB_THREADS * PB_ITEMS;
    for (int64_t t0 = (int64_t)blockIdx.x * TILE; t0 < nnz; t0 += (int64_t)gridDim.x * TILE) {
        for (int64_t d = threadIdx.x; d < nb; d += blockDim.x) s_run[d] = 0;
        __syncthreads();
        // every entry is read once: its indices and value stay in registers across the
        // reservation
        uint32_t packed[PB_ITEMS];  // bucket << 16 | rank in the tile's run
        uint64_t key[PB_ITEMS];     // row in the bucket << (mb + pb) | minor << pb | position
        typename std::conditional<HAS_VAL, VT, char>::type val[PB_ITEMS];
        int64_t mjs[PB_ITEMS], mns[PB_ITEMS];
        // all loads first, so that they are in flight together (the shared-memory atomics below
        // would otherwise keep each entry's loads behind the previous entry's atomic)
#pragma unroll
        for (int q = 0; q < PB_ITEMS; ++q) {
            const int64_t e = t0 + (int64_t)q * PB_THREADS + threadIdx.x;
            mjs[q] = -1;
            mns[q] = 0;
            if (e < nnz) {
                src.get(e, mjs[q], mns[q]);
                if constexpr (HAS_VAL) val[q] = vals_in[e];
            }
        }
#pragma unroll
        for (int q = 0; q < PB_ITEMS; ++q) {
            const int64_t e = t0 + (int64_t)q * PB_THREADS + threadIdx.x;
            const int64_t mj = mjs[q], mn = mns[q];
            const bool in = (uint64_t)mj < (uint64_t)major_n;
            const uint32_t d = (uint32_t)(in ? mj >> cs : nb - 1);
            const uint64_t lrow = in ? (uint64_t)(mj - ((int64_t)d << cs)) : 0;
            // the minor index masked to its field, so that an index outside the matrix cannot
            // reach the row bits
            key[q] = shl64(lrow, co.mb + co.pb) | ((((uint64_t)mn) & low_mask(co.mb)) << co.pb) | (uint64_t)e;
            packed[q] = e < nnz ? (d << 16) | atomicAdd(&s_run[d], 1u) : 0u;
        }
        __syncthreads();
        // one reservation per bucket the tile touches; eight independent atomics in flight
        // per thread (cfill starts at the buckets' first slots)
        for (int64_t d0 = threadIdx.x; d0 < nb; d0 += (int64_t)PB_THREADS * 8) {
            uint32_t c[8], got[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t d = d0 + (int64_t)u * PB_THREADS;
                c[u] = d < nb ? s_run[d] : 0;
                got[u] = c[u] ? atomicAdd(&cfill[d], c[u]) : 0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (c[u]) s_run[d0 + (int64_t)u * PB_THREADS] = got[u];
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PB_ITEMS; ++q) {
            const int64_t e = t0 + (int64_t)q * PB_THREADS + threadIdx.x;
            if (e < nnz) {
                const uint32_t slot = s_run[packed[q] >> 16] + (packed[q] & 0xffffu);
                if constexpr (HAS_VAL) store_rec(rec1 + slot, key[q], val[q]);
                else rec1[slot] = Rec<VT>{key[q]};
            }
        }
        __syncthreads();
    }
}

// Dynamic shared memory of fine_kernel: the staged keys and values, then row offsets and
// fill counters for 2^cs rows.
template <class VT> inline size_t fine_smem_bytes(int cs) {
    return (size_t)stage_entries<VT>() * (8 + carried_size<VT>()) + (((size_t)2 << cs) + 2) * sizeof(uint32_t);
}

// CTA per coarse bucket: rows counted and scanned in shared memory (the row pointers), then
// the bucket's entries placed in row order -- into shared memory when the bucket fits the
// staging (rows of up to 16 entries sorted there by a thread, up to 256 by a warp, longer
// ones copied out for cta_kernel), else into key2 / val2 (read back in this kernel: plain
// pointers, no read-only cache path) with rows of more than 16 entries listed for
// warp_kernel and cta_kernel.
template <class VT, class Emit>
__global__ void __launch_bounds__(PC_THREADS, 2)
fine_kernel(int64_t major_n, Coarse co, const uint32_t *__restrict__ cstart, const Rec<VT> *__restrict__ rec1,
            uint64_t *key2, VT *val2, uint32_t *__restrict__ start, uint32_t *__restrict__ list,
            uint32_t *__restrict__ counters, Emit emit) {
    constexpr bool HAS_VAL = !std::is_same<VT, NoValue>::value;
    const int cs = co.cs;
    const int64_t nb = co.nb;
    const int rshift = co.mb + co.pb;  // the row inside the bucket sits above minor and position
    const PackedEmit<Emit> pemit{emit, co.mb, co.pb};
    constexpr int STAGE = stage_entries<VT>();
    constexpr int ITEMS = ROWS_MAX / PC_THREADS;
    extern __shared__ __align__(16) unsigned char dsm[];
    uint64_t *s_key = (uint64_t *)dsm;
    VT *s_val = (VT *)(dsm + (size_t)STAGE * 8);
    uint32_t *s_off = (uint32_t *)(dsm + (size_t)STAGE * (8 + carried_size<VT>()));
    const int rmax = 1 << cs;
    uint32_t *s_fill = s_off + rmax + 1;  // counts, then fill cursors, then the warp row list
    __shared__ uint32_t s_warp[PC_THREADS / 32];
    __shared__ uint32_t s_nlist, s_long;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t bk = blockIdx.x; bk < nb; bk += gridDim.x) {
        const uint32_t B0 = cstart[bk], B1 = cstart[bk + 1];
        const uint32_t E = B1 - B0;
        const bool invalid = bk == nb - 1;
        const int64_t row0 = invalid ? major_n : bk << cs;
        const int64_t rspan = major_n - row0 < (int64_t)rmax ? major_n - row0 : (int64_t)rmax;
        const int R = invalid ? 1 : (int)rspan;
        const bool staged = E <= (uint32_t)STAGE;
        for (int j = threadIdx.x; j < R; j += PC_THREADS) s_fill[j] = 0;
        if (threadIdx.x == 0) {
            s_nlist = 0;
            s_long = 0;
        }
        __syncthreads();
#pragma unroll 4
        for (uint32_t i = B0 + threadIdx.x; i < B1; i += PC_THREADS)
            atomicAdd(&s_fill[(uint32_t)shr64(rec1[i].key, rshift)], 1u);
        __syncthreads();
        // exclusive scan of the R row counts: each thread takes ITEMS consecutive rows
        uint32_t v[ITEMS], sum = 0;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const int j = threadIdx.x * ITEMS + q;
            v[q] = j < R ? s_fill[j] : 0;
            sum += v[q];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t wsum = lane < PC_THREADS / 32 ? s_warp[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wsum, o);
                if (lane >= o) wsum += y;
            }
            if (lane < PC_THREADS / 32) s_warp[lane] = wsum;
        }
        __syncthreads();
        uint32_t run = (warp ? s_warp[warp - 1] : 0) + x - sum;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const int j = threadIdx.x * ITEMS + q;
            if (j < R) s_off[j] = run;
            run += v[q];
        }
        if (threadIdx.x == 0) s_off[R] = E;
        __syncthreads();
        for (int j = threadIdx.x; j < R; j += PC_THREADS) {
            const uint32_t first = B0 + s_off[j];
            start[row0 + j] = first;
            emit.pointer(row0 + j, first);
            s_fill[j] = 0;
            if (s_off[j + 1] - s_off[j] > (uint32_t)WARP_MAX) s_long = 1;
        }
        if (invalid && threadIdx.x == 0) start[major_n + 1] = B1;
        __syncthreads();
        if (staged) {
#pragma unroll 4
            for (uint32_t i = B0 + threadIdx.x; i < B1; i += PC_THREADS) {
                const Rec<VT> r = rec1[i];
                const uint32_t row = (uint32_t)shr64(r.key, rshift);
                const uint32_t slot = s_off[row] + atomicAdd(&s_fill[row], 1u);
                s_key[slot] = r.key;
                if constexpr (HAS_VAL) s_val[slot] = r.val;
            }
            __syncthreads();
            if (s_long) {  // rows for cta_kernel read their (plain) keys from key2
                for (uint32_t j = threadIdx.x; j < E; j += PC_THREADS)
                    key2[B0 + j] = canonical_key(s_key[j], co.mb, co.pb);
            }
            __syncthreads();  // s_fill becomes the list of warp-sized rows
            for (int j0 = 0; j0 < R; j0 += PC_THREADS) {
                const int j = j0 + threadIdx.x;
                const bool valid = j < R;
                uint32_t len = 0;
                if (valid) {
                    len = s_off[j + 1] - s_off[j];
                    if (len <= (uint32_t)SMALL)
                        sort_short_row(s_key + s_off[j], HAS_VAL ? s_val + s_off[j] : nullptr, B0 + s_off[j], len,
                                       (uint64_t)(row0 + j), pemit);
                    else if (len <= (uint32_t)WARP_MAX)
                        s_fill[atomicAdd(&s_nlist, 1u)] = (uint32_t)j;
                }
                list_long_rows(valid && len > (uint32_t)WARP_MAX, len, (uint32_t)(row0 + j), major_n, list,
                               counters);
            }
            __syncthreads();
            for (uint32_t q = warp; q < s_nlist; q += PC_THREADS / 32) {
                const uint32_t j = s_fill[q];
                const uint32_t o = s_off[j], len = s_off[j + 1] - o;
                for (uint32_t t = lane; t < len; t += 32) {
                    const uint64_t kt = s_key[o + t];
                    uint32_t rank = 0;
                    for (uint32_t u = 0; u < len; ++u) rank += s_key[o + u] < kt ? 1u : 0u;
                    emit_one(pemit, B0 + o + rank, (uint64_t)(row0 + j), kt, HAS_VAL ? s_val + o : nullptr, t);
                }
            }
        } else {
            for (uint32_t i = B0 + threadIdx.x; i < B1; i += PC_THREADS) {
                const Rec<VT> r = rec1[i];
                const uint32_t row = (uint32_t)shr64(r.key, rshift);
                const uint32_t slot = B0 + s_off[row] + atomicAdd(&s_fill[row], 1u);
                key2[slot] = canonical_key(r.key, co.mb, co.pb);
                if constexpr (HAS_VAL) val2[slot] = r.val;
            }
            __syncthreads();
            for (int j0 = 0; j0 < R; j0 += PC_THREADS) {
                const int j = j0 + threadIdx.x;
                const bool valid = j < R;
                uint32_t len = 0;
                if (valid) {
                    const uint32_t b = B0 + s_off[j];
                    len = s_off[j + 1] - s_off[j];
                    if (len <= (uint32_t)SMALL)
                        sort_short_row(key2 + b, HAS_VAL ? val2 + b : nullptr, b, len, (uint64_t)(row0 + j), emit);
                }
                list_long_rows(valid, len, (uint32_t)(row0 + j), major_n, list, counters);
            }
        }
        __syncthreads();
    }
}

// ---- staged two-level form -------------------------------------------------
//
// Pass C with one CTA of 1024 threads per SM that copies its next bucket into shared memory
// with cp.async while it sorts the current one, so that the loads stay in flight across the
// pass's barriers instead of waiting behind them.  It places a bucket's records by 16-bit
// indices in shared memory, sorts each row's indices there and writes the bucket's output in
// order with coalesced stores; a bucket larger than its buffer takes the global path of
// fine_kernel.  The row pointers and the output are the same as fine_kernel's.

constexpr int ST_THREADS = 1024;
constexpr int FS_MAXI = 8;                   // pass C: at most 8 staged records per thread
constexpr int STAGE_ROW_AVG = 8;             // pass C staged while rows average at most 8 entries
// Pass C staged: a thread sorts rows of up to 8 entries in place, a warp rows of 9 to 256.  (A
// 16-key in-place thread sort, which at this kernel's 64 registers runs mostly from spilled
// registers, left rows of 9 to 16 entries unsorted and corrupted the index array on GB300; the
// warp sort takes those rows.)
constexpr int STAGE_SMALL = 8;

// The CTA copies the bytes [src, src + bytes) to dst, both 16-byte aligned, in 16-byte
// pieces; a last partial piece reads only its own bytes and zero-fills the rest.
__device__ __forceinline__ void copy_to_shared(void *dst, const void *src, uint64_t bytes) {
    const uint64_t pieces = (bytes + 15) >> 4;
    for (uint64_t c = threadIdx.x; c < pieces; c += blockDim.x) {
        const uint64_t left = bytes - (c << 4);
        cp_async16((char *)dst + (c << 4), (const char *)src + (c << 4), left < 16 ? (uint32_t)left : 16u);
    }
}

// Rank-counting sort, by the records' keys, of the N or fewer record indices of one row
// (idx[0 .. len)), in place: all indices are read before any is written (volatile reads, so
// that none is read again after the stores).
template <class R, int N>
__device__ __forceinline__ void sort_idx_registers(const R *rec, uint16_t *idx, uint32_t len) {
    const volatile uint16_t *vidx = idx;
    uint64_t k[N];
    uint32_t ix[N / 2];  // two 16-bit indices per register
#pragma unroll
    for (int j = 0; j < N; j += 2) {
        const uint32_t a = (uint32_t)j < len ? vidx[j] : 0u, b = (uint32_t)j + 1 < len ? vidx[j + 1] : 0u;
        ix[j / 2] = a | (b << 16);
        k[j] = (uint32_t)j < len ? rec[a].key : ~0ull;
        k[j + 1] = (uint32_t)j + 1 < len ? rec[b].key : ~0ull;
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
        if ((uint32_t)j >= len) break;
        uint32_t rank = 0;
#pragma unroll
        for (int q = 0; q < N; ++q) rank += k[q] < k[j] ? 1u : 0u;
        idx[rank] = (uint16_t)(ix[j / 2] >> (16 * (j & 1)));
    }
}
template <class R> __device__ __forceinline__ void sort_idx_short(const R *rec, uint16_t *idx, uint32_t len) {
    if (len <= 1) return;
    if (len <= 4) sort_idx_registers<R, 4>(rec, idx, len);
    else sort_idx_registers<R, STAGE_SMALL>(rec, idx, len);
}
// A warp sorts the record indices of one row of up to WARP_MAX entries in place: each lane
// holds up to 8 keys, and every key is compared with the row's keys broadcast 32 at a time.
template <class R> __device__ __forceinline__ void sort_idx_warp(const R *rec, uint16_t *idx, uint32_t len, int lane) {
    constexpr int P = WARP_MAX / 32;
    uint64_t k[P];
    uint32_t ix[P], rank[P];
#pragma unroll
    for (int m = 0; m < P; ++m) {
        const uint32_t t = (uint32_t)(m * 32 + lane);
        ix[m] = t < len ? idx[t] : 0u;
        k[m] = t < len ? rec[ix[m]].key : ~0ull;
        rank[m] = 0;
    }
#pragma unroll
    for (int g = 0; g < P; ++g) {
        if ((uint32_t)(g * 32) >= len) break;  // uniform across the warp
        for (int l = 0; l < 32; ++l) {
            const uint64_t kl = __shfl_sync(0xffffffffu, k[g], l);
#pragma unroll
            for (int m = 0; m < P; ++m)
                if ((uint32_t)(m * 32) < len) rank[m] += kl < k[m] ? 1u : 0u;
        }
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < P; ++m) {
        const uint32_t t = (uint32_t)(m * 32 + lane);
        if (t < len) idx[rank[m]] = (uint16_t)ix[m];
    }
    __syncwarp();
}

// Pass C's buffer: the most records per bucket whose two buffers and index array fit beside
// the row offsets and counters (a multiple of 16, at most FS_MAXI * ST_THREADS).
template <class VT> inline int fine_stage_cap(int cs, size_t smem_max) {
    const size_t rows = (((size_t)2 << cs) + 2) * sizeof(uint32_t);
    if (smem_max <= rows) return 0;
    int64_t c = (int64_t)((smem_max - rows) / (2 * sizeof(Rec<VT>) + sizeof(uint16_t)));
    c &= ~(int64_t)15;
    return (int)(c > FS_MAXI * ST_THREADS ? FS_MAXI * ST_THREADS : c);
}
template <class VT> inline size_t fine_stage_smem(int cs, int cap) {
    return 2 * (size_t)cap * sizeof(Rec<VT>) + (size_t)cap * sizeof(uint16_t) + (((size_t)2 << cs) + 2) * sizeof(uint32_t);
}

// Pass C, staged: one CTA per SM takes buckets from a queue (counters[2]) and copies the
// next bucket's records into shared memory while it sorts the current one.  Rows are
// counted, scanned (the row pointers) and placed as record indices; rows of up to 16
// entries are sorted by a thread, up to 256 by a warp, longer ones listed for cta_kernel;
// then the bucket's output is written in order.  A bucket of more than `cap` entries takes
// fine_kernel's global path (rows placed into key2 / val2, then sorted there or listed).
template <class VT, class Emit>
__global__ void __launch_bounds__(ST_THREADS, 1)
fine_stage_kernel(int64_t major_n, Coarse co, int cap, const uint32_t *__restrict__ cstart,
                  const Rec<VT> *__restrict__ rec1, uint64_t *key2, VT *val2, uint32_t *__restrict__ start,
                  uint32_t *__restrict__ list, uint32_t *__restrict__ counters, Emit emit) {
    constexpr bool HAS_VAL = !std::is_same<VT, NoValue>::value;
    constexpr int ITEMS = ROWS_MAX / ST_THREADS;
    const int cs = co.cs;
    const int64_t nb = co.nb;
    const int rshift = co.mb + co.pb;
    const PackedEmit<Emit> pemit{emit, co.mb, co.pb};
    extern __shared__ __align__(16) unsigned char dsm[];
    Rec<VT> *s_buf = (Rec<VT> *)dsm;  // two buffers of cap records
    uint16_t *s_idx = (uint16_t *)(s_buf + 2 * (size_t)cap);
    uint32_t *s_off = (uint32_t *)(s_idx + cap);
    const int rmax = 1 << cs;
    uint32_t *s_cnt = s_off + rmax + 1;  // row counts; then fill cursors (global path) or the warp row list
    __shared__ uint32_t s_warp[ST_THREADS / 32];
    __shared__ uint32_t s_nlist, s_long;
    __shared__ int64_t s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t bk = blockIdx.x;
    if (bk < nb) {
        const uint32_t b0 = cstart[bk], e = cstart[bk + 1] - b0;
        if (e <= (uint32_t)cap) copy_to_shared(s_buf, rec1 + b0, (uint64_t)e * sizeof(Rec<VT>));
    }
    cp_async_commit();
    for (int b = 0; bk < nb; b ^= 1) {
        const uint32_t B0 = cstart[bk], B1 = cstart[bk + 1];
        const uint32_t E = B1 - B0;
        const bool invalid = bk == nb - 1;
        const int64_t row0 = invalid ? major_n : bk << cs;
        const int64_t rspan = major_n - row0 < (int64_t)rmax ? major_n - row0 : (int64_t)rmax;
        const int R = invalid ? 1 : (int)rspan;
        const bool staged = E <= (uint32_t)cap;
        for (int j = threadIdx.x; j < R; j += ST_THREADS) s_cnt[j] = 0;
        if (threadIdx.x == 0) {
            s_next = (int64_t)gridDim.x + atomicAdd(&counters[2], 1u);
            s_nlist = 0;
            s_long = 0;
        }
        __syncthreads();
        const int64_t nx = s_next;
        // the other buffer was last read before the previous bucket's final barrier
        if (nx < nb) {
            const uint32_t b0 = cstart[nx], e = cstart[nx + 1] - b0;
            if (e <= (uint32_t)cap)
                copy_to_shared(s_buf + (size_t)(b ^ 1) * cap, rec1 + b0, (uint64_t)e * sizeof(Rec<VT>));
        }
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();  // bucket bk's records in shared memory
        const Rec<VT> *s_rec = s_buf + (size_t)b * cap;
        uint32_t pr[FS_MAXI];  // row << 16 | arrival rank in the row
        if (staged) {
#pragma unroll
            for (int q = 0; q < FS_MAXI; ++q) {
                const uint32_t j = (uint32_t)(q * ST_THREADS) + threadIdx.x;
                pr[q] = 0;
                if (j < E) {
                    const uint32_t row = (uint32_t)shr64(s_rec[j].key, rshift);
                    pr[q] = (row << 16) | atomicAdd(&s_cnt[row], 1u);
                }
            }
        } else {
#pragma unroll 4
            for (uint32_t i = B0 + threadIdx.x; i < B1; i += ST_THREADS)
                atomicAdd(&s_cnt[(uint32_t)shr64(rec1[i].key, rshift)], 1u);
        }
        __syncthreads();
        // exclusive scan of the R row counts: each thread takes ITEMS consecutive rows
        uint32_t v[ITEMS], sum = 0;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const int j = threadIdx.x * ITEMS + q;
            v[q] = j < R ? s_cnt[j] : 0;
            sum += v[q];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t wsum = s_warp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wsum, o);
                if (lane >= o) wsum += y;
            }
            s_warp[lane] = wsum;
        }
        __syncthreads();
        uint32_t run = (warp ? s_warp[warp - 1] : 0) + x - sum;
#pragma unroll
        for (int q = 0; q < ITEMS; ++q) {
            const int j = threadIdx.x * ITEMS + q;
            if (j < R) s_off[j] = run;
            run += v[q];
        }
        if (threadIdx.x == 0) s_off[R] = E;
        __syncthreads();
        for (int j = threadIdx.x; j < R; j += ST_THREADS) {
            const uint32_t first = B0 + s_off[j];
            start[row0 + j] = first;
            emit.pointer(row0 + j, first);
            if (!staged) s_cnt[j] = 0;  // the global path's fill cursors
            if (s_off[j + 1] - s_off[j] > (uint32_t)WARP_MAX) s_long = 1;
        }
        if (invalid && threadIdx.x == 0) start[major_n + 1] = B1;
        if (staged) {
            // s_off is complete since the scan; the row counts are no longer read
#pragma unroll
            for (int q = 0; q < FS_MAXI; ++q) {
                const uint32_t j = (uint32_t)(q * ST_THREADS) + threadIdx.x;
                if (j < E) s_idx[s_off[pr[q] >> 16] + (pr[q] & 0xffffu)] = (uint16_t)j;
            }
            __syncthreads();
            if (s_long) {  // rows for cta_kernel read their (plain) keys from key2
                for (uint32_t p = threadIdx.x; p < E; p += ST_THREADS)
                    key2[B0 + p] = canonical_key(s_rec[s_idx[p]].key, co.mb, co.pb);
            }
            for (int j0 = 0; j0 < R; j0 += ST_THREADS) {
                const int j = j0 + threadIdx.x;
                const bool valid = j < R;
                uint32_t len = 0;
                if (valid) {
                    const uint32_t o = s_off[j];
                    len = s_off[j + 1] - o;
                    if (len <= (uint32_t)STAGE_SMALL) sort_idx_short(s_rec, s_idx + o, len);
                    else if (len <= (uint32_t)WARP_MAX) s_cnt[atomicAdd(&s_nlist, 1u)] = (uint32_t)j;
                }
                list_long_rows(valid && len > (uint32_t)WARP_MAX, len, (uint32_t)(row0 + j), major_n, list,
                               counters);
            }
            __syncthreads();
            if (s_nlist) {  // uniform
                for (uint32_t q = warp; q < s_nlist; q += ST_THREADS / 32) {
                    const uint32_t j = s_cnt[q];
                    const uint32_t o = s_off[j];
                    sort_idx_warp(s_rec, s_idx + o, s_off[j + 1] - o, lane);
                }
                __syncthreads();
            }
            // the bucket's output in order (rows listed for cta_kernel are rewritten by it)
            for (uint32_t p = threadIdx.x; p < E; p += ST_THREADS) {
                const Rec<VT> r = s_rec[s_idx[p]];
                const uint64_t row = (uint64_t)row0 + shr64(r.key, rshift);
                if constexpr (HAS_VAL) pemit.put(B0 + p, row, r.key, r.val);
                else pemit.gather(B0 + p, row, r.key);
            }
        } else {
            __syncthreads();  // the fill cursors are zero
            for (uint32_t i = B0 + threadIdx.x; i < B1; i += ST_THREADS) {
                const Rec<VT> r = rec1[i];
                const uint32_t row = (uint32_t)shr64(r.key, rshift);
                const uint32_t slot = B0 + s_off[row] + atomicAdd(&s_cnt[row], 1u);
                key2[slot] = canonical_key(r.key, co.mb, co.pb);
                if constexpr (HAS_VAL) val2[slot] = r.val;
            }
            __syncthreads();
            for (int j0 = 0; j0 < R; j0 += ST_THREADS) {
                const int j = j0 + threadIdx.x;
                const bool valid = j < R;
                uint32_t len = 0;
                if (valid) {
                    const uint32_t b2 = B0 + s_off[j];
                    len = s_off[j + 1] - s_off[j];
                    if (len <= (uint32_t)SMALL)
                        sort_short_row(key2 + b2, HAS_VAL ? val2 + b2 : nullptr, b2, len, (uint64_t)(row0 + j), emit);
                }
                list_long_rows(valid, len, (uint32_t)(row0 + j), major_n, list, counters);
            }
        }
        __syncthreads();
        bk = nx;
    }
    cp_async_wait<0>();
}

// ---- one-level form (more rows than the coarse buckets cover) --------------

template <class Src>
__global__ void count_kernel(Src src, int64_t nnz, int64_t major_n, uint32_t *__restrict__ cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t mj = src.major(i);
        atomicAdd(&cnt[(uint64_t)mj < (uint64_t)major_n ? mj : major_n], 1u);
    }
}

template <class Src>
__global__ void place_kernel(Src src, int64_t nnz, int64_t major_n, const uint32_t *__restrict__ start,
                             uint32_t *__restrict__ fill, uint64_t *__restrict__ keys) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t mj, mn;
        src.get(i, mj, mn);
        const int64_t r = (uint64_t)mj < (uint64_t)major_n ? mj : major_n;
        keys[(uint64_t)start[r] + atomicAdd(&fill[r], 1u)] = ((uint64_t)(uint32_t)mn << 32) | (uint32_t)i;
    }
}

template <class Emit>
__global__ void small_kernel(int64_t major_n, const uint32_t *__restrict__ start, const uint64_t *__restrict__ keys,
                             uint32_t *__restrict__ list, uint32_t *__restrict__ counters, Emit emit) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r0 = (int64_t)blockIdx.x * blockDim.x; r0 <= major_n; r0 += stride) {
        const int64_t r = r0 + threadIdx.x;
        const bool valid = r <= major_n;
        uint32_t len = 0;
        if (valid) {
            const uint32_t b = start[r];
            len = start[r + 1] - b;
            emit.pointer(r, b);
            if (len <= (uint32_t)SMALL) sort_short_row<Emit, NoValue>(keys + b, nullptr, b, len, (uint64_t)r, emit);
        }
        list_long_rows(valid, len, (uint32_t)r, major_n, list, counters);
    }
}

// ---- long rows (both forms) --------------------------------------------------

// Warp per listed row of (SMALL, WARP_MAX] entries: the row's keys in shared memory, each
// entry's rank = the number of smaller keys; values (when carried) move with their keys.
template <class VT, class Emit>
__global__ void __launch_bounds__(WARP_CTA_THREADS)
warp_kernel(const uint32_t *__restrict__ start, const uint64_t *__restrict__ keys, const VT *__restrict__ vals,
            const uint32_t *__restrict__ list, const uint32_t *__restrict__ counters, Emit emit) {
    __shared__ uint64_t s[WARP_CTA_THREADS / 32][WARP_MAX];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t nlisted = counters[0];
    const int64_t warps = (int64_t)gridDim.x * (WARP_CTA_THREADS / 32);
    for (int64_t q = (int64_t)blockIdx.x * (WARP_CTA_THREADS / 32) + w; q < nlisted; q += warps) {
        const uint32_t r = list[q];
        const uint32_t b = start[r], len = start[r + 1] - b;
        for (uint32_t j = lane; j < len; j += 32) s[w][j] = keys[b + j];
        __syncwarp();
        for (uint32_t j = lane; j < len; j += 32) {
            const uint64_t kj = s[w][j];
            uint32_t rank = 0;
            for (uint32_t t = 0; t < len; ++t) rank += s[w][t] < kj ? 1u : 0u;
            emit_one(emit, b + rank, (uint64_t)r, kj, vals, b + j);
        }
        __syncwarp();
    }
}

__device__ __forceinline__ void bitonic_shared(uint64_t *s, uint32_t P) {
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = s[i], c = s[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > c) == up) {
                        s[i] = c;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// One CTA merges the sorted runs A (na) and B (nb) into out (distinct keys).
__device__ __forceinline__ void merge_runs(const uint64_t *A, uint32_t na, const uint64_t *B, uint32_t nb,
                                           uint64_t *out) {
    const uint32_t total = na + nb;
    for (uint32_t t0 = 0; t0 < total; t0 += blockDim.x * MERGE_ITEMS) {
        const uint32_t d0 = t0 + threadIdx.x * MERGE_ITEMS;
        if (d0 >= total) continue;
        uint32_t lo = d0 > nb ? d0 - nb : 0, hi = d0 < na ? d0 : na;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (A[mid] < B[d0 - 1 - mid]) lo = mid + 1;
            else hi = mid;
        }
        uint32_t i = lo, j = d0 - lo;
        for (int q = 0; q < MERGE_ITEMS && d0 + q < total; ++q) {
            if (j >= nb || (i < na && A[i] < B[j])) out[d0 + q] = A[i++];
            else out[d0 + q] = B[j++];
        }
    }
}

// CTA per listed row of more than WARP_MAX entries.  Rows of up to RANK_MAX keys: each key's
// position is the number of smaller keys in the row (shared memory, two barriers per row);
// up to CTA_TILE keys: bitonic sort in shared memory; longer rows sorted in CTA_TILE chunks,
// then merged pairwise between keys and scratch (the row's own range in each).  Values are
// gathered by input position.
template <class Emit>
__global__ void __launch_bounds__(CTA_THREADS)
cta_kernel(int64_t major_n, const uint32_t *__restrict__ start, uint64_t *keys, uint64_t *scratch,
           const uint32_t *__restrict__ list, const uint32_t *__restrict__ counters, Emit emit) {
    extern __shared__ __align__(16) uint64_t s[];  // CTA_TILE keys
    const uint32_t nlisted = counters[1];
    for (uint32_t q = blockIdx.x; q < nlisted; q += gridDim.x) {
        const uint32_t r = list[major_n - q];
        const uint32_t b = start[r], len = start[r + 1] - b;
        if (len <= (uint32_t)RANK_MAX) {  // keys are distinct (they hold the input position)
            for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) s[j] = keys[b + j];
            __syncthreads();
            for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) {
                const uint64_t kj = s[j];
                uint32_t rank = 0;
#pragma unroll 4
                for (uint32_t u = 0; u < len; ++u) rank += s[u] < kj ? 1u : 0u;
                emit.gather(b + rank, (uint64_t)r, kj);
            }
            __syncthreads();
            continue;
        }
        for (uint32_t c0 = 0; c0 < len; c0 += CTA_TILE) {
            const uint32_t n = len - c0 < (uint32_t)CTA_TILE ? len - c0 : (uint32_t)CTA_TILE;
            uint32_t P = 2;
            while (P < n) P <<= 1;
            for (uint32_t j = threadIdx.x; j < P; j += blockDim.x) s[j] = j < n ? keys[b + c0 + j] : ~0ull;
            __syncthreads();
            bitonic_shared(s, P);
            if (len <= (uint32_t)CTA_TILE) {
                for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) emit.gather(b + j, (uint64_t)r, s[j]);
            } else {
                for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) keys[b + c0 + j] = s[j];
            }
            __syncthreads();
        }
        if (len <= (uint32_t)CTA_TILE) continue;
        uint64_t *src = keys + b, *dst = scratch + b;
        for (uint32_t w = CTA_TILE; w < len; w <<= 1) {
            for (uint32_t lo = 0; lo < len; lo += 2 * w) {
                const uint32_t na = len - lo < w ? len - lo : w;
                const uint32_t rest = len - lo - na;
                const uint32_t nb = rest < w ? rest : w;
                merge_runs(src + lo, na, src + lo + na, nb, dst + lo);
            }
            __syncthreads();
            uint64_t *t = src; src = dst; dst = t;
        }
        for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) emit.gather(b + j, (uint64_t)r, src[j]);
        __syncthreads();
    }
}

template <class Emit>
int launch_cta(cudaStream_t s, int64_t major_n, const uint32_t *start, uint64_t *keys, uint64_t *scratch,
               const uint32_t *list, const uint32_t *counters, const Emit &emit) {
    const size_t smem = (size_t)CTA_TILE * sizeof(uint64_t);
    int rc = check_cuda(cudaFuncSetAttribute(cta_kernel<Emit>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "bucket: cta_kernel shared memory");
    if (rc) return rc;
    cta_kernel<Emit><<<152, CTA_THREADS, smem, s>>>(major_n, start, keys, scratch, list, counters, emit);
    return check_cuda(cudaGetLastError(), "bucket cta_kernel");
}

inline unsigned grid_for(int64_t n, int64_t per_cta, int64_t cap) {
    int64_t b = ceil_div(n, per_cta);
    if (b > cap) b = cap;
    return (unsigned)(b > 0 ? b : 1);
}

// The whole sort.  vals_in: the values to carry (VT = NoValue: none).  scan(s, in, out, n,
// bsums) is the library's exclusive scan of uint32.
template <class Src, class VT, class Emit, class Scan>
int sort(cudaStream_t s, int64_t major_n, int64_t minor_n, int64_t nnz, const Src &src, const VT *vals_in,
         const Emit &emit, void *ws, Scan scan, size_t sc_tile) {
    constexpr size_t VS = std::is_same<VT, NoValue>::value ? 0 : sizeof(VT);
    static_assert(sizeof(Rec<VT>) == rec_size(VS), "record size of the layout");
    const Layout L = layout(major_n, minor_n, nnz, VS, sc_tile);
    char *w = (char *)ws;
    uint32_t *cnt = (uint32_t *)(w + L.cnt), *start = (uint32_t *)(w + L.start);
    uint32_t *bsums = (uint32_t *)(w + L.bsums), *list = (uint32_t *)(w + L.list);
    uint32_t *counters = (uint32_t *)(w + L.counters);
    uint64_t *key1 = (uint64_t *)(w + L.key1), *key2 = (uint64_t *)(w + L.key2);
    int rc = check_cuda(cudaMemsetAsync(cnt, 0, (size_t)L.ncnt * sizeof(uint32_t), s), "bucket: clear");
    if (!rc) rc = check_cuda(cudaMemsetAsync(counters, 0, 4 * sizeof(uint32_t), s), "bucket: clear");
    if (rc) return rc;
    const int64_t cap = 152 * 16;
    if (L.co.ok) {
        const Coarse co = L.co;
        uint32_t *cstart = (uint32_t *)(w + L.cstart);
        Rec<VT> *rec1 = (Rec<VT> *)(w + L.rec1);
        VT *val2 = VS ? (VT *)(w + L.val2) : nullptr;
        const bool staged = get_sort_staged() != 0;
        int sms = 0, optin = 0;
        if (staged) {
            int dev = 0;
            rc = check_cuda(cudaGetDevice(&dev), "bucket: device");
            if (!rc) rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "bucket: SMs");
            if (!rc)
                rc = check_cuda(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                                "bucket: shared memory");
            if (rc) return rc;
        }
        // dynamic shared memory the staged kernels may take (their static arrays stay below 512 B)
        const size_t smax = optin > 1024 ? (size_t)optin - 512 : 0;
        // the counting pass: six CTAs of 32 KB histograms per SM, each flushing its counts once
        if (nnz > 0)
            coarse_count_kernel<Src><<<grid_for(nnz, PB_THREADS * PB_ITEMS, staged ? (int64_t)sms * 6 : cap),
                                       PB_THREADS, 0, s>>>(src, nnz, major_n, co.cs, co.nb, cnt);
        rc = check_cuda(cudaGetLastError(), "bucket coarse_count_kernel");
        if (!rc) rc = scan(s, cnt, cstart, co.nb + 1, bsums);  // cstart[nb] = nnz
        // the fill cursors start at the buckets' first slots
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(cnt, cstart, (size_t)(co.nb + 1) * sizeof(uint32_t),
                                            cudaMemcpyDeviceToDevice, s),
                            "bucket: cursors");
        if (rc) return rc;
        if (nnz > 0)
            coarse_place_kernel<Src, VT><<<grid_for(nnz, PB_THREADS * PB_ITEMS, cap), PB_THREADS, 0, s>>>(
                src, vals_in, nnz, major_n, co, cnt, rec1);
        // the staged pass C copies whole 16-byte-aligned records (conversions carry values); it
        // pays where rows are short (thread-sorted): with longer rows, most entries are sorted by
        // warps, whose uneven work two CTAs per SM overlap better (power-law rows averaging 16
        // entries: 1151 us staged against 671 us)
        const bool short_rows = nnz <= STAGE_ROW_AVG * major_n;
        const int fcap = staged && short_rows && sizeof(Rec<VT>) % 16 == 0 ? fine_stage_cap<VT>(co.cs, smax) : 0;
        if (fcap >= ST_THREADS) {
            const size_t sm = fine_stage_smem<VT>(co.cs, fcap);
            rc = check_cuda(cudaFuncSetAttribute(fine_stage_kernel<VT, Emit>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                            "bucket: fine_stage_kernel shared memory");
            if (rc) return rc;
            fine_stage_kernel<VT, Emit><<<(unsigned)(co.nb < sms ? co.nb : sms), ST_THREADS, sm, s>>>(
                major_n, co, fcap, cstart, rec1, key2, val2, start, list, counters, emit);
            warp_kernel<VT, Emit><<<152 * 8, WARP_CTA_THREADS, 0, s>>>(start, key2, val2, list, counters, emit);
            rc = launch_cta(s, major_n, start, key2, key1, list, counters, emit);
            if (rc) return rc;
            return check_cuda(cudaGetLastError(), "bucket sort kernels");
        }
        const size_t smem = fine_smem_bytes<VT>(co.cs);
        rc = check_cuda(cudaFuncSetAttribute(fine_kernel<VT, Emit>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem),
                        "bucket: fine_kernel shared memory");
        if (rc) return rc;
        fine_kernel<VT, Emit><<<grid_for(co.nb, 1, 152 * 2), PC_THREADS, smem, s>>>(
            major_n, co, cstart, rec1, key2, val2, start, list, counters, emit);
        warp_kernel<VT, Emit><<<152 * 8, WARP_CTA_THREADS, 0, s>>>(start, key2, val2, list, counters, emit);
        rc = launch_cta(s, major_n, start, key2, key1, list, counters, emit);
        if (rc) return rc;
        return check_cuda(cudaGetLastError(), "bucket sort kernels");
    }
    if (nnz > 0) count_kernel<Src><<<grid_for(nnz, 256, cap), 256, 0, s>>>(src, nnz, major_n, cnt);
    rc = check_cuda(cudaGetLastError(), "bucket count_kernel");
    if (!rc) rc = scan(s, cnt, start, major_n + 2, bsums);
    if (!rc) rc = check_cuda(cudaMemsetAsync(cnt, 0, (size_t)L.ncnt * sizeof(uint32_t), s), "bucket: clear");
    if (rc) return rc;
    if (nnz > 0) place_kernel<Src><<<grid_for(nnz, 256, cap), 256, 0, s>>>(src, nnz, major_n, start, cnt, key1);
    small_kernel<Emit><<<grid_for(major_n + 1, 256, 152 * 32), 256, 0, s>>>(major_n, start, key1, list, counters,
                                                                             emit);
    warp_kernel<NoValue, Emit><<<152 * 8, WARP_CTA_THREADS, 0, s>>>(start, key1, nullptr, list, counters, emit);
    rc = launch_cta(s, major_n, start, key1, key2, list, counters, emit);
    if (rc) return rc;
    return check_cuda(cudaGetLastError(), "bucket sort kernels");
}

}  // namespace bucket
}  // namespace gsa
