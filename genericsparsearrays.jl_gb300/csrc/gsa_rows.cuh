// Row-gather device code shared by the plain kernel (gsa_rowblock.cu) and the grouped
// kernel (gsa_batch.cu): sums over row segments, G lanes per row for a warp's rows.
#pragma once

#include <type_traits>

#include "gsa_internal.cuh"

namespace gsa {

constexpr int RB_THREADS = 128;
constexpr int RB_WARPS = RB_THREADS / 32;
constexpr int G1_AVG = 6;       // a thread per row while a warp's rows average <= 6 entries
constexpr int PLAN_LEN = 32;    // with a plan, rows longer than this go to the plan's warps
constexpr int UNROLL = 4;       // entries per lane in flight on a plan warp
constexpr int CHUNK = 512;      // entries per plan warp (longer rows are cut into chunks)

// Offsets into idx / val: the unsigned type of the index width.  Int32 row pointers
// hold offsets below 2^31, so 32-bit arithmetic is exact there and j + U*S cannot wrap;
// narrow offsets keep the thread-per-row path within 32 registers.
template <typename I> using Off = typename std::make_unsigned<I>::type;

// acc[c] += sum over j = jb, jb+S, ... < je of conj?(a_j) * op(B)(idx_j, c0 + c), in j order.
// An index outside [base, base + inner_n) never leads to a read outside B: the
// unsigned offset idx_j - base is compared with inner_n (saturated to the offset width).
// Entries a one-lane-per-row pass loads ahead of its multiply-adds (4 measured 60.5 us on
// the 2048^2 Laplacian F64/Int32 SpMV against 61.8 us with 1, at the same 32 registers).
#ifndef GSA_G1_UNROLL
#define GSA_G1_UNROLL 4
#endif
// The same for rows shared by several lanes (2 measured 738 us on a 16-column F64 SpMM of the
// 2048^2 Laplacian against 850 us with 4).
#ifndef GSA_GN_UNROLL
#define GSA_GN_UNROLL 2
#endif

// The same for Float64 with B.pairs: op(B)(i, c0 + c) read two columns per 16-byte load (c0
// and c even), the multiply-adds in the same order as accumulate_range's.
template <typename I, int KC, int S, int U>
__device__ __forceinline__ void accumulate_pairs(const CompressedArgs<double, I> &a, const DenseIn<double> &B,
                                                 Off<I> jb, Off<I> je, int64_t c0, int64_t k,
                                                 double (&acc)[KC]) {
    using O = Off<I>;
    const I *__restrict__ idx = a.idx;
    const double *__restrict__ val = a.val;
    const O inner = sizeof(O) == 8 ? (O)a.inner_n
                                   : (O)(a.inner_n < 0xffffffffLL ? a.inner_n : 0xffffffffLL);
    const O base = (O)a.base;
    auto row_fma = [&](O ci, double av) {
        const bool ok = ci < inner;
        const double *q = B.p + (int64_t)(ok ? ci : 0) * B.rs + c0;
#pragma unroll
        for (int c = 0; c < KC; c += 2) {
            if (c0 + c + 1 < k) {
                const double2 x = ok ? __ldg(reinterpret_cast<const double2 *>(q + c)) : make_double2(0.0, 0.0);
                acc[c] = fma(av, x.x, acc[c]);
                acc[c + 1] = fma(av, x.y, acc[c + 1]);
            } else if (c0 + c < k) {
                acc[c] = fma(av, ok ? __ldg(q + c) : 0.0, acc[c]);
            }
        }
    };
    O j = jb;
    if (U > 1) {
        for (; j + (O)((U - 1) * S) < je; j += U * S) {
            O ci[U];
            double av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ci[u] = (O)idx[j + u * S] - base;
                av[u] = val[j + u * S];
            }
#pragma unroll
            for (int u = 0; u < U; ++u) row_fma(ci[u], av[u]);
        }
    }
    for (; j < je; j += S) row_fma((O)idx[j] - base, val[j]);
}

template <typename V, typename I, int KC, int S, int U>
__device__ __forceinline__ void accumulate_range(const CompressedArgs<V, I> &a, const DenseIn<V> &B,
                                                 Off<I> jb, Off<I> je, int64_t c0, int64_t k,
                                                 V (&acc)[KC]) {
    // only in the 4- and 8-column kernels (what a row-major B takes): compiled into the
    // 2-column kernel of a column-major B it cost 8 registers and 12 % of the Laplacian SpMM
    if constexpr (std::is_same<V, double>::value && KC >= 4) {
        if (B.pairs) {
            accumulate_pairs<I, KC, S, U>(a, B, jb, je, c0, k, acc);
            return;
        }
    }
    using O = Off<I>;
    const I *__restrict__ idx = a.idx;
    const V *__restrict__ val = a.val;
    const O inner = sizeof(O) == 8 ? (O)a.inner_n
                                   : (O)(a.inner_n < 0xffffffffLL ? a.inner_n : 0xffffffffLL);
    const O base = (O)a.base;
    O j = jb;
    if (U > 1) {
        for (; j + (O)((U - 1) * S) < je; j += U * S) {
            O ci[U];
            V av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ci[u] = (O)idx[j + u * S] - base;
                av[u] = conj_if(val[j + u * S], a.conjA);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = ci[u] < inner;
#pragma unroll
                for (int c = 0; c < KC; ++c)
                    if (KC == 1 || c0 + c < k) {
                        const V xv = ok ? B.at((int64_t)ci[u], c0 + c) : VT<V>::zero();
                        acc[c] = mac(acc[c], av[u], xv);
                    }
            }
        }
    }
    for (; j < je; j += S) {
        const O c1 = (O)idx[j] - base;
        const bool ok = c1 < inner;
        const V av = conj_if(val[j], a.conjA);
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (KC == 1 || c0 + c < k) {
                const V xv = ok ? B.at((int64_t)c1, c0 + c) : VT<V>::zero();
                acc[c] = mac(acc[c], av, xv);
            }
    }
}

// The 32 rows of one warp (lane l owns row row0 + l, entries [b, e)), G lanes per
// row: in each of G passes the warp's 32/G groups take one row each, the group's
// lanes stride the row, a width-G shuffle tree reduces, the group's first lane
// stores.  G = 1 is a thread per row.
template <typename V, typename I, int KC, int G>
__device__ __forceinline__ void warp_rows(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                          const DenseOut<V> &C, int64_t c0, int64_t row0, Off<I> b,
                                          Off<I> e, int skip) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    constexpr int RPP = 32 / G;  // rows per pass
#pragma unroll 1
    for (int p = 0; p < G; ++p) {
        const int q = p * RPP + lane / G;
        const O qb = G == 1 ? b : (O)__shfl_sync(0xffffffffu, b, q);
        const O qe = G == 1 ? e : (O)__shfl_sync(0xffffffffu, e, q);
        const int qskip = G == 1 ? skip : __shfl_sync(0xffffffffu, skip, q);
        V acc[KC];
#pragma unroll
        for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
        accumulate_range<V, I, KC, G, (G == 1 ? GSA_G1_UNROLL : GSA_GN_UNROLL)>(a, B, qb + (O)(lane % G), qe, c0, k,
                                                                              acc);
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

// The device view of a plan (gsa_plan): planned outer entries, their chunks, the skip
// mask the row blocks read, and (gather only) the counters and partial sums of rows of
// more than one chunk.
struct PlanRows {
    int64_t nlong, nchunks;
    const int64_t *row;        // nlong: outer index of each planned entry
    const int32_t *first;      // nlong: its first chunk
    const int32_t *count;      // nlong: its number of chunks
    const int32_t *chunk_slot; // nchunks: the planned entry (slot) a chunk belongs to
    const uint32_t *skip_mask; // ceil(outer_n / 32): bit l of word w marks entry 32w + l as planned
    int *done;                 // nlong * ncg counters, zero before the launch, reset after
    void *partial;             // nchunks * k values
};

// The device view of one chunk set of a plan (no counters or partials yet).
inline PlanRows plan_rows(const gsa_chunk_set &c) {
    PlanRows L{};
    L.nlong = c.nlong;
    L.nchunks = c.nchunks;
    L.row = c.row;
    L.first = c.first;
    L.count = c.count;
    L.chunk_slot = c.chunk_slot;
    L.skip_mask = c.skip_mask;
    return L;
}

// The extents [b, e) of one warp's 32 outer entries starting at row0 (a multiple of 32),
// clamped to [0, nnz] (a malformed pointer never leads outside idx/val); entries the plan
// takes (bit l of skip_mask[row0 / 32]) get an empty extent and skip = 1.  Returns the
// average extent of the warp's remaining entries.
template <typename V, typename I>
__device__ __forceinline__ int64_t warp_extent(const CompressedArgs<V, I> &a, int64_t row0,
                                               const uint32_t *__restrict__ skip_mask, Off<I> &b,
                                               Off<I> &e, int &skip) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const int64_t r = row0 + lane;
    b = 0;
    e = 0;
    if (r < a.outer_n) {
        const O nz = (O)a.nnz, base = (O)a.base;
        b = (O)__ldg(a.ptr + r) - base;
        e = (O)__ldg(a.ptr + r + 1) - base;
        b = b < nz ? b : nz;
        e = e < nz ? e : nz;
        e = e < b ? b : e;
    }
    skip = 0;
    int64_t total;
    if (skip_mask) {
        skip = (int)((__ldg(skip_mask + (row0 >> 5)) >> lane) & 1u);
        if (skip) e = b;
        // the entries left here are at most CHUNK long: their sum fits 32 bits
        total = (int64_t)__reduce_add_sync(0xffffffffu, (unsigned)(e - b));
    } else {
        total = (int64_t)__shfl_sync(0xffffffffu, e, 31) - (int64_t)__shfl_sync(0xffffffffu, b, 0);
    }
    return total >> 5;
}

// Calls f(std::integral_constant<int, G>) for G the power of two with G * g1_avg covering
// avg (1 when avg is at most g1_avg, 32 at most).
template <typename F>
__device__ __forceinline__ void dispatch_lanes(int64_t avg, int g1_avg, F &&f) {
    if (avg <= g1_avg) f(std::integral_constant<int, 1>{});
    else if (avg <= 2 * g1_avg) f(std::integral_constant<int, 2>{});
    else if (avg <= 4 * g1_avg) f(std::integral_constant<int, 4>{});
    else if (avg <= 8 * g1_avg) f(std::integral_constant<int, 8>{});
    else if (avg <= 16 * g1_avg) f(std::integral_constant<int, 16>{});
    else f(std::integral_constant<int, 32>{});
}

// One warp's 32 rows starting at row0 (a multiple of 32), G lanes per row (see
// dispatch_lanes); rows the plan takes are left to its warps.
template <typename V, typename I, int KC>
__device__ __forceinline__ void warp_unit(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                          const DenseOut<V> &C, int64_t c0, int64_t row0,
                                          const uint32_t *__restrict__ skip_mask, int g1_avg = G1_AVG) {
    Off<I> b, e;
    int skip;
    const int64_t avg = warp_extent(a, row0, skip_mask, b, e, skip);
    dispatch_lanes(avg, g1_avg, [&](auto g) {
        warp_rows<V, I, KC, decltype(g)::value>(a, k, B, C, c0, row0, b, e, skip);
    });
}

// ---------------------------------------------------------------------------
// Bin order (a plan's): within each segment of rows, rows grouped by the multiply-adds each
// of their lanes does; warp w of the order takes 32 / G consecutive rows of its group, G
// lanes each, so the lanes of a warp do equal work.

// Position range [pos0, pend) of warp w of a bin order and its lanes per row.
__device__ __forceinline__ void bin_warp(const gsa_bin_order &bv, int64_t w, int64_t &pos0, int64_t &pend, int &G) {
    const int gi = __ldg(bv.warp_group + w);
    const int64_t first_warp = __ldg(bv.groups + 4 * gi), pos = __ldg(bv.groups + 4 * gi + 1);
    pend = __ldg(bv.groups + 4 * gi + 2);
    G = (int)__ldg(bv.groups + 4 * gi + 3);
    pos0 = pos + (w - first_warp) * (32 / G);
}

// Row at position i of a bin order and its extent [b, e), clamped to [0, nnz].
template <typename V, typename I>
__device__ __forceinline__ int64_t bin_row(const CompressedArgs<V, I> &a, const gsa_bin_order &bv, int64_t i,
                                           Off<I> &b, Off<I> &e) {
    using O = Off<I>;
    const int64_t row = __ldg(bv.perm + i);
    if (row >= a.outer_n) {
        b = e = 0;
        return row;
    }
    const O nz = (O)a.nnz, base = (O)a.base;
    b = (O)__ldg(a.ptr + row) - base;
    e = (O)__ldg(a.ptr + row + 1) - base;
    b = b < nz ? b : nz;
    e = e < nz ? e : nz;
    e = e < b ? b : e;
    return row;
}

template <typename V, typename I, int KC, int G>
__device__ __forceinline__ void binned_rows(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                            const DenseOut<V> &C, int64_t c0, int64_t pos0, int64_t pend,
                                            const gsa_bin_order &bv) {
    using O = Off<I>;
    const int lane = threadIdx.x & 31;
    const int64_t i = pos0 + lane / G;
    const bool valid = i < pend;
    int64_t row = 0;
    O b = 0, e = 0;
    if (valid) row = bin_row(a, bv, i, b, e);
    V acc[KC];
#pragma unroll
    for (int c = 0; c < KC; ++c) acc[c] = VT<V>::zero();
    accumulate_range<V, I, KC, G, 2>(a, B, b + (O)(lane % G), e, c0, k, acc);
    if (G > 1) {
#pragma unroll
        for (int c = 0; c < KC; ++c) {
#pragma unroll
            for (int m = G / 2; m > 0; m >>= 1) acc[c] = add(acc[c], shfl_xor(acc[c], m, G));
        }
    }
    if (lane % G == 0 && valid && row < a.outer_n) {
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (KC == 1 || c0 + c < k) C.store(row, c0 + c, acc[c]);
    }
}

// Warp w of the bin order (w < bv.nwarps).
template <typename V, typename I, int KC>
__device__ __forceinline__ void binned_warp(const CompressedArgs<V, I> &a, int64_t k, const DenseIn<V> &B,
                                            const DenseOut<V> &C, int64_t c0, int64_t w,
                                            const gsa_bin_order &bv) {
    int64_t pos0, pend;
    int G;
    bin_warp(bv, w, pos0, pend, G);
    dispatch_lanes(G, 1, [&](auto g) {  // G is a power of two: picks exactly G lanes
        binned_rows<V, I, KC, decltype(g)::value>(a, k, B, C, c0, pos0, pend, bv);
    });
}

}  // namespace gsa
