// Internal definitions shared by the libgsa translation units: value types,
// arithmetic in the reference's conventions, dense-operand accessors, error
// reporting and the dtype x itype dispatch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <math.h>

#include <type_traits>

#include "../../include/gsa.h"

// A plan (gsa_plan_create), device arrays in one allocation.  In the natural order of row
// blocks, outer entries of more than 512 stored entries, and those of more than 32 that
// are over 4x the average of their aligned group of 32, are cut into chunks of 512 (the
// `nat` set, marked in its skip_mask).  When lengths vary so much inside groups of 32
// that lanes would idle, the plan also has a bin order: within each segment of 32768
// consecutive outer entries, the entries of at most 512 sorted by the number of
// multiply-adds each of their lanes does and grouped by their lanes per entry, so that the
// lanes of a warp do equal work and a segment's entries are read close together in time;
// longer ones are chunked (`bin`).
struct gsa_chunk_set {
    int64_t nlong = 0, nchunks = 0;       // chunked entries and their chunks
    const int64_t *row = nullptr;         // outer index of each chunked entry
    const int32_t *first = nullptr;       // its first chunk
    const int32_t *count = nullptr;       // its number of chunks
    const int32_t *chunk_slot = nullptr;  // the chunked entry a chunk belongs to
    const uint32_t *skip_mask = nullptr;  // bit per outer entry, 1 = chunked
};
// A plan's bin order as the kernels read it (also copied into the plan's device memory,
// for grouped launches whose items point at it).  A group is one lanes-per-entry class of
// one segment.
struct gsa_bin_order {
    int64_t nwarps;             // warps of the bin order
    const int32_t *perm;        // outer entries, group by group (extents from the pointers)
    const int32_t *warp_group;  // group of each warp
    const int64_t *groups;      // per group: first warp, first position, end position, lanes
};
struct gsa_plan {
    int64_t outer_n = 0, nnz = 0, max_len = 0;
    int64_t nplanned = 0;                 // entries the plan takes out of the natural order
    gsa_chunk_set nat;                    // natural order: > 512, or > 32 and over 4x the group
    gsa_chunk_set bin;                    // bin order: > 512 only
    // bin order (nbin_warps > 0)
    int64_t nbin_warps = 0;
    gsa_bin_order order{};                // its arrays (device pointers)
    const gsa_bin_order *bin_view = nullptr;  // device copy of `order`
    void *mem = nullptr;
    // COO plans (gsa_coo_plan_create): row pointers of a row-sorted COO (owned), the rest of
    // the plan describing them; coo_sorted = 0 leaves the COO kernel in charge
    int coo = 0, coo_sorted = 0;
    void *coo_ptr = nullptr;
};

namespace gsa {

// ---------------------------------------------------------------------------
// Value types.  Complex numbers are (re, im) pairs aligned to twice the real
// size, matching Julia's ComplexF32/ComplexF64 arrays and numpy/torch complex.
struct alignas(8) cf32 { float re, im; };
struct alignas(16) cf64 { double re, im; };

template <typename V> struct VT;
template <> struct VT<float> {
    static constexpr bool is_complex = false;
    __host__ __device__ static float zero() { return 0.0f; }
};
template <> struct VT<double> {
    static constexpr bool is_complex = false;
    __host__ __device__ static double zero() { return 0.0; }
};
template <> struct VT<cf32> {
    static constexpr bool is_complex = true;
    __host__ __device__ static cf32 zero() { return cf32{0.0f, 0.0f}; }
};
template <> struct VT<cf64> {
    static constexpr bool is_complex = true;
    __host__ __device__ static cf64 zero() { return cf64{0.0, 0.0}; }
};
template <> struct VT<int32_t> {
    static constexpr bool is_complex = false;
    __host__ __device__ static int32_t zero() { return 0; }
};
template <> struct VT<int64_t> {
    static constexpr bool is_complex = false;
    __host__ __device__ static int64_t zero() { return 0; }
};

// Arithmetic.  Integers wrap (Julia's Int32/Int64 semantics).  Floating-point
// multiply-adds are explicit fused multiply-adds and nothing else is contracted (the
// library builds with -fmad=false): GB300 issues about two FP64 FMAs per clock per SM,
// so FP64 products are bound by that pipe about as much as by HBM, and one FMA per
// real multiply-add (four per complex one) halves the FP64 instructions of a
// multiply-then-add.  Results stay within the double-double oracle's tolerance; a row
// summed in the same order gives the same bits in every kernel.
__host__ __device__ __forceinline__ float add(float a, float b) { return a + b; }
__host__ __device__ __forceinline__ double add(double a, double b) { return a + b; }
__host__ __device__ __forceinline__ cf32 add(cf32 a, cf32 b) { return cf32{a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cf64 add(cf64 a, cf64 b) { return cf64{a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ int32_t add(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a + (uint32_t)b);
}
__host__ __device__ __forceinline__ int64_t add(int64_t a, int64_t b) {
    return (int64_t)((uint64_t)a + (uint64_t)b);
}

__host__ __device__ __forceinline__ float mul(float a, float b) { return a * b; }
__host__ __device__ __forceinline__ double mul(double a, double b) { return a * b; }
// (ar + i ai)(br + i bi) = (ar br - ai bi) + i (ar bi + ai br), one product of each
// part fused into the other's add
__host__ __device__ __forceinline__ cf32 mul(cf32 a, cf32 b) {
    return cf32{fmaf(a.re, b.re, -(a.im * b.im)), fmaf(a.re, b.im, a.im * b.re)};
}
__host__ __device__ __forceinline__ cf64 mul(cf64 a, cf64 b) {
    return cf64{fma(a.re, b.re, -(a.im * b.im)), fma(a.re, b.im, a.im * b.re)};
}
__host__ __device__ __forceinline__ int32_t mul(int32_t a, int32_t b) {
    return (int32_t)((uint32_t)a * (uint32_t)b);
}
__host__ __device__ __forceinline__ int64_t mul(int64_t a, int64_t b) {
    return (int64_t)((uint64_t)a * (uint64_t)b);
}

// acc + a * b
__host__ __device__ __forceinline__ float mac(float acc, float a, float b) { return fmaf(a, b, acc); }
__host__ __device__ __forceinline__ double mac(double acc, double a, double b) { return fma(a, b, acc); }
__host__ __device__ __forceinline__ cf32 mac(cf32 acc, cf32 a, cf32 b) {
    return cf32{fmaf(-a.im, b.im, fmaf(a.re, b.re, acc.re)), fmaf(a.im, b.re, fmaf(a.re, b.im, acc.im))};
}
__host__ __device__ __forceinline__ cf64 mac(cf64 acc, cf64 a, cf64 b) {
    return cf64{fma(-a.im, b.im, fma(a.re, b.re, acc.re)), fma(a.im, b.re, fma(a.re, b.im, acc.im))};
}
__host__ __device__ __forceinline__ int32_t mac(int32_t acc, int32_t a, int32_t b) { return add(acc, mul(a, b)); }
__host__ __device__ __forceinline__ int64_t mac(int64_t acc, int64_t a, int64_t b) { return add(acc, mul(a, b)); }

// Conjugation flips the sign bit of the imaginary part with an integer XOR: the same
// bits as negation, without an FP add (a negated double would take the FP64 pipe).
__host__ __device__ __forceinline__ float flip_sign_if(float x, bool c) {
#ifdef __CUDA_ARCH__
    return __int_as_float(__float_as_int(x) ^ ((int)c << 31));
#else
    return c ? -x : x;
#endif
}
__host__ __device__ __forceinline__ double flip_sign_if(double x, bool c) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)c << 63));
#else
    return c ? -x : x;
#endif
}
template <typename V> __host__ __device__ __forceinline__ V conj_if(V a, bool c) { return a; }
template <> __host__ __device__ __forceinline__ cf32 conj_if(cf32 a, bool c) {
    return cf32{a.re, flip_sign_if(a.im, c)};
}
template <> __host__ __device__ __forceinline__ cf64 conj_if(cf64 a, bool c) {
    return cf64{a.re, flip_sign_if(a.im, c)};
}

template <typename V> __host__ __device__ __forceinline__ bool is_zero(V a) { return a == V(0); }
template <> __host__ __device__ __forceinline__ bool is_zero(cf32 a) { return a.re == 0.0f && a.im == 0.0f; }
template <> __host__ __device__ __forceinline__ bool is_zero(cf64 a) { return a.re == 0.0 && a.im == 0.0; }
template <typename V> __host__ __device__ __forceinline__ bool is_one(V a) { return a == V(1); }
template <> __host__ __device__ __forceinline__ bool is_one(cf32 a) { return a.re == 1.0f && a.im == 0.0f; }
template <> __host__ __device__ __forceinline__ bool is_one(cf64 a) { return a.re == 1.0 && a.im == 0.0; }

// Read-only (non-coherent) loads for operands the kernel never writes.
template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }
template <> __device__ __forceinline__ cf32 ldg(const cf32 *p) {
    float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return cf32{v.x, v.y};
}
template <> __device__ __forceinline__ cf64 ldg(const cf64 *p) {
    double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return cf64{v.x, v.y};
}

// Loads that bypass L1 (L2 is coherent across SMs): data other CTAs wrote during the kernel.
template <typename T> __device__ __forceinline__ T ld_coherent(const T *p) { return __ldcg(p); }
template <> __device__ __forceinline__ cf32 ld_coherent(const cf32 *p) {
    float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    return cf32{v.x, v.y};
}
template <> __device__ __forceinline__ cf64 ld_coherent(const cf64 *p) {
    double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
    return cf64{v.x, v.y};
}

// Asynchronous 16-byte copies global -> shared (cp.async, L1 bypassed): `bytes` (0..16) are
// read from src and the rest of the 16 zero-filled; both addresses 16-byte aligned.  A
// thread's copies are grouped by commit, and wait_group<N> returns once at most N of its
// groups are still in flight (the copies become visible to other threads at the next barrier).
__device__ __forceinline__ void cp_async16(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Streaming loads for data read exactly once (matrix entries): evict-first.
template <typename T> __device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }
template <> __device__ __forceinline__ cf32 ld_stream(const cf32 *p) {
    float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    return cf32{v.x, v.y};
}
template <> __device__ __forceinline__ cf64 ld_stream(const cf64 *p) {
    double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    return cf64{v.x, v.y};
}

// Atomic accumulate (complex: one atomic per component).
__device__ __forceinline__ void atomic_add(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add(double *p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add(cf32 *p, cf32 v) {
    atomicAdd(&p->re, v.re);
    atomicAdd(&p->im, v.im);
}
__device__ __forceinline__ void atomic_add(cf64 *p, cf64 v) {
    atomicAdd(&p->re, v.re);
    atomicAdd(&p->im, v.im);
}
__device__ __forceinline__ void atomic_add(int32_t *p, int32_t v) { atomicAdd((int *)p, (int)v); }
__device__ __forceinline__ void atomic_add(int64_t *p, int64_t v) {
    atomicAdd((unsigned long long *)p, (unsigned long long)v);
}

// Warp shuffles for every value type.
template <typename V> __device__ __forceinline__ V shfl_up(V v, int d) {
    return __shfl_up_sync(0xffffffffu, v, d);
}
template <> __device__ __forceinline__ cf32 shfl_up(cf32 v, int d) {
    return cf32{__shfl_up_sync(0xffffffffu, v.re, d), __shfl_up_sync(0xffffffffu, v.im, d)};
}
template <> __device__ __forceinline__ cf64 shfl_up(cf64 v, int d) {
    return cf64{__shfl_up_sync(0xffffffffu, v.re, d), __shfl_up_sync(0xffffffffu, v.im, d)};
}
template <typename V> __device__ __forceinline__ V shfl_xor(V v, int m, int w = 32) {
    return __shfl_xor_sync(0xffffffffu, v, m, w);
}
template <> __device__ __forceinline__ cf32 shfl_xor(cf32 v, int m, int w) {
    return cf32{__shfl_xor_sync(0xffffffffu, v.re, m, w), __shfl_xor_sync(0xffffffffu, v.im, m, w)};
}
template <> __device__ __forceinline__ cf64 shfl_xor(cf64 v, int m, int w) {
    return cf64{__shfl_xor_sync(0xffffffffu, v.re, m, w), __shfl_xor_sync(0xffffffffu, v.im, m, w)};
}
template <typename V> __device__ __forceinline__ V shfl_down(V v, int d) {
    return __shfl_down_sync(0xffffffffu, v, d);
}
template <> __device__ __forceinline__ cf32 shfl_down(cf32 v, int d) {
    return cf32{__shfl_down_sync(0xffffffffu, v.re, d), __shfl_down_sync(0xffffffffu, v.im, d)};
}
template <> __device__ __forceinline__ cf64 shfl_down(cf64 v, int d) {
    return cf64{__shfl_down_sync(0xffffffffu, v.re, d), __shfl_down_sync(0xffffffffu, v.im, d)};
}

// ---------------------------------------------------------------------------
// Dense operand views.  op(B)(i, c) = B[i*rs + c*cs], conjugated if conj.
// pairs: the caller checked that op(B)(i, c) and op(B)(i, c + 1) for even c are one aligned
// 16-byte piece (Float64, unit column stride, even row stride, 16-byte aligned p), so a
// thread's columns of one row may be read two at a time (by kernels of 4 or 8 columns).
template <typename V> struct DenseIn {
    const V *p;
    int64_t rs, cs;
    bool conj;
    bool pairs = false;
    __device__ __forceinline__ V at(int64_t i, int64_t c) const {
        return conj_if(ldg(p + i * rs + c * cs), conj);
    }
};

// Whether a Float64 operand's rows can be read two columns at a time (see DenseIn::pairs).
template <typename V> inline bool pairs_ok(const DenseIn<V> &B) {
    return std::is_same<V, double>::value && B.cs == 1 && (B.rs & 1) == 0 && ((uintptr_t)B.p & 15) == 0;
}

// 0 + x without an FP add: x, except that -0 becomes +0 (integer compare and select,
// so the FP64 pipe is not used).
__device__ __forceinline__ float zero_plus(float x) {
    return __float_as_int(x) == (int)0x80000000u ? 0.0f : x;
}
__device__ __forceinline__ double zero_plus(double x) {
    return __double_as_longlong(x) == (long long)0x8000000000000000ull ? 0.0 : x;
}
__device__ __forceinline__ cf32 zero_plus(cf32 x) { return cf32{zero_plus(x.re), zero_plus(x.im)}; }
__device__ __forceinline__ cf64 zero_plus(cf64 x) { return cf64{zero_plus(x.re), zero_plus(x.im)}; }
__device__ __forceinline__ int32_t zero_plus(int32_t x) { return x; }
__device__ __forceinline__ int64_t zero_plus(int64_t x) { return x; }

// C column-major with leading dimension ld; beta handled per LinearAlgebra's
// _rmul_or_fill!: beta == 1 keeps C, beta == 0 overwrites without reading (the
// reference then adds into the zero it filled: 0 + t).  alpha == 1 of a real type is
// not multiplied (t * 1 == t for every t), which saves an FP64 instruction per row.
template <typename V> struct DenseOut {
    V *p;
    int64_t ld;
    V alpha, beta;
    int beta_mode;  // 0: beta == 0, 1: beta == 1, 2: general
    bool alpha_one; // alpha == 1 and V is real
    // C[i, c] = beta*C[i, c] + acc*alpha
    __device__ __forceinline__ void store(int64_t i, int64_t c, V acc) const {
        V *q = p + i * 1 + c * ld;
        V t = alpha_one ? acc : mul(acc, alpha);
        if (beta_mode == 0) *q = zero_plus(t);
        else if (beta_mode == 1) *q = add(*q, t);
        else *q = mac(t, *q, beta);
    }
    // C[i, c] += v (for values already multiplied by alpha)
    __device__ __forceinline__ void accumulate(int64_t i, int64_t c, V v) const {
        V *q = p + i + c * ld;
        *q = add(*q, v);
    }
};

template <typename V> inline int beta_mode_of(V beta) {
    return is_zero(beta) ? 0 : (is_one(beta) ? 1 : 2);
}
template <typename V> __host__ __device__ inline bool alpha_one_of(V alpha) {
    return !VT<V>::is_complex && is_one(alpha);
}

// ---------------------------------------------------------------------------
// Errors.
void set_error(const char *fmt, ...);
int fail(int status, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);

// Optional events recorded right before and after the main compute kernel of the next
// calls on this host thread (set by gsa_set_kernel_timer).
void timer_before(cudaStream_t s);
void timer_after(cudaStream_t s);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Exclusive scan of n uint32 counts (in and out may be the same array); block_sums holds
// scan_block_sums(n) entries of scratch.
constexpr int SCAN_TILE = 4096;
inline int64_t scan_block_sums(int64_t n) { return ceil_div(n, SCAN_TILE) + 1; }
int scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *block_sums);

// Stable LSD radix sort of (uint64 key, uint32 payload) pairs over the low total_bits bits
// (8-bit digits).  Fill the buffers radix_sort_inputs returns, then sort; the sorted pairs
// are in *keys_out / *perm_out (one of the workspace's two buffer pairs).
size_t radix_sort_workspace(int64_t n);
void radix_sort_inputs(void *ws, int64_t n, uint64_t **keys, uint32_t **perm);
int radix_sort_pairs(cudaStream_t s, void *ws, int64_t n, int total_bits, uint64_t **keys_out, uint32_t **perm_out);
int radix_bits_for(int64_t count);  // bits that values 0 .. count - 1 need

// Scratch of one call: the caller's buffer, or a stream-ordered allocation freed on the
// same stream when the call returns.
struct Workspace {
    void *p = nullptr;
    size_t bytes = 0;
    bool owned = false;
    cudaStream_t s = nullptr;
    int acquire(cudaStream_t stream, void *user, size_t user_bytes, size_t need) {
        s = stream;
        if (need == 0) { p = user; bytes = user_bytes; return GSA_OK; }
        if (user) {
            if (user_bytes < need)
                return fail(GSA_ERR_INVALID_ARG, "workspace of %zu bytes is smaller than the %zu needed",
                            user_bytes, need);
            p = user;
            bytes = user_bytes;
            return GSA_OK;
        }
        cudaError_t e = cudaMallocAsync(&p, need, stream);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(GSA_ERR_ALLOC, "stream-ordered workspace allocation of %zu bytes failed: %s",
                        need, cudaGetErrorString(e));
        }
        owned = true;
        bytes = need;
        return GSA_OK;
    }
    ~Workspace() {
        if (owned && p) cudaFreeAsync(p, s);
    }
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Splits one workspace into aligned sub-buffers.
struct Carver {
    char *base;
    size_t off = 0;
    explicit Carver(void *b) : base((char *)b) {}
    template <typename T> T *take(size_t count) {
        off = align_up(off, 256);
        T *p = base ? (T *)(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
    // the offset of the next region (256-byte aligned), for layouts that record offsets
    template <typename T> size_t reserve(size_t count) {
        off = align_up(off, 256);
        const size_t at = off;
        off += count * sizeof(T);
        return at;
    }
};

// Dispatch helpers: call F.template operator()<V, I>() for runtime codes.
template <typename F> int dispatch_vi(int dtype, int itype, F &&f) {
    if (itype == GSA_IDX32) {
        switch (dtype) {
        case GSA_F32: return f.template operator()<float, int32_t>();
        case GSA_F64: return f.template operator()<double, int32_t>();
        case GSA_C32: return f.template operator()<cf32, int32_t>();
        case GSA_C64: return f.template operator()<cf64, int32_t>();
        case GSA_I32: return f.template operator()<int32_t, int32_t>();
        case GSA_I64: return f.template operator()<int64_t, int32_t>();
        }
    } else if (itype == GSA_IDX64) {
        switch (dtype) {
        case GSA_F32: return f.template operator()<float, int64_t>();
        case GSA_F64: return f.template operator()<double, int64_t>();
        case GSA_C32: return f.template operator()<cf32, int64_t>();
        case GSA_C64: return f.template operator()<cf64, int64_t>();
        case GSA_I32: return f.template operator()<int32_t, int64_t>();
        case GSA_I64: return f.template operator()<int64_t, int64_t>();
        }
    }
    return fail(GSA_ERR_UNSUPPORTED, "unsupported dtype %d / itype %d", dtype, itype);
}

inline size_t dtype_size(int dtype) {
    switch (dtype) {
    case GSA_F32: return 4;
    case GSA_F64: return 8;
    case GSA_C32: return 8;
    case GSA_C64: return 16;
    case GSA_I32: return 4;
    case GSA_I64: return 8;
    }
    return 0;
}
inline size_t itype_size(int itype) { return itype == GSA_IDX32 ? 4 : (itype == GSA_IDX64 ? 8 : 0); }

// ---------------------------------------------------------------------------
// Kernel entry points implemented in the .cu files (host-side launchers).

// Arguments of one sparse x dense product in "compressed outer" form: the
// outer dimension is the one ptr compresses (rows for CSR, columns for CSC).
template <typename V, typename I> struct CompressedArgs {
    int64_t outer_n;   // number of compressed rows/columns
    int64_t inner_n;   // range of idx (entries outside it are skipped, never read or written)
    int64_t nnz;
    const I *ptr;      // outer_n + 1 entries
    const I *idx;      // nnz entries
    const V *val;      // nnz entries
    int base;
    bool conjA;
};

// Gather: out[o, c] = beta*out[o, c] + alpha * sum_j conj?(val_j) * op(B)(idx_j, c)
template <typename V, typename I>
int launch_gather(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                  DenseOut<V> C, int algo, const ::gsa_plan *plan, void *ws, size_t ws_bytes);
template <typename V, typename I>
size_t gather_workspace_size(int64_t outer_n, int64_t nnz, int64_t k, int algo, const ::gsa_plan *plan);

using Plan = ::gsa_plan;
int plan_create(cudaStream_t s, int itype, int64_t outer_n, int64_t nnz, const void *ptr, int base, Plan *p);
// Row pointers of a COO whose row indices are non-decreasing and within [base, base + m)
// (sets *sorted = 0 otherwise; synchronizes s).
int coo_row_pointers(cudaStream_t s, int itype, int64_t m, int64_t nnz, const void *rowind, int base,
                     void *ptr_out, int *sorted);

// Row-block gather (thread per short row; long rows by warp, or by plan chunks): the default.
template <typename V, typename I>
int launch_rowblock(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                    DenseOut<V> C, const Plan *plan, void *ws, size_t ws_bytes);
size_t rowblock_workspace_size(const Plan *plan, size_t vsize, int64_t k);
// Persistent bulk-copy pipelined merge-path SpMV (k = 1): GSA_ALGO_PIPE.
template <typename V, typename I>
int launch_spmv_pipe(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B, DenseOut<V> C,
                     void *ws, size_t ws_bytes);
template <typename V, typename I> size_t spmv_pipe_workspace_size(int64_t outer_n, int64_t nnz);
// The same product with its carry slots in a static device array (no allocation).
template <typename V, typename I>
int launch_spmv_noalloc(cudaStream_t s, const CompressedArgs<V, I> &a, DenseIn<V> B, DenseOut<V> C);
// Reads and clears the device error word of bounded waits (synchronizes s).
int read_pipe_error(cudaStream_t s, int *out);
void set_pipe_threads(int t);
int get_pipe_threads();
void set_wait_limit(uint32_t polls);  // polls of a bounded wait before it gives up
uint32_t get_wait_limit();
void set_spmm_columns(int c);   // 0 (by value size), 1, 2, 4 or 8
int get_spmm_columns();
void set_plan_natural(int v);   // 1: row blocks in natural order even where a plan bins them
int get_plan_natural();
void set_stage_rows(int v);     // 1: thread-per-row warps stage their span with 16-byte loads
int get_stage_rows();
void set_x_pairs(int v);        // 1 (default): Float64 row-major B read two columns per load
int get_x_pairs();
void set_sort_staged(int v);    // 1 (default): the bucket sort's staged passes (one CTA per SM)
int get_sort_staged();

// Scatter: out[idx_j, c] += conj?(val_j) * (op(B)(o, c) * alpha), after the beta pass.
// ALGO_MERGE: merge-path tiles (workspace: tile coordinates); otherwise outer blocks with
// an optional plan (no workspace).
template <typename V, typename I>
int launch_scatter(cudaStream_t s, const CompressedArgs<V, I> &a, int64_t k, DenseIn<V> B,
                   DenseOut<V> C, int64_t out_rows, int algo, const Plan *plan, void *ws,
                   size_t ws_bytes);
template <typename V, typename I>
size_t scatter_workspace_size(int64_t outer_n, int64_t nnz, int64_t k, int algo);

// dot(x, op(A), y) for fmt 0 CSR, 1 CSC (optional plan), 2 COO; the scalar is copied to
// result_host and the stream synchronized.
template <typename V, typename I>
size_t dot_workspace_size(int fmt, int64_t outer_n, const Plan *plan);
template <typename V, typename I>
int launch_dot(cudaStream_t s, int fmt, int opA, int64_t m, int64_t n, int64_t nnz, const I *p0,
               const I *p1, const V *val, int base, const V *x, const V *y, const Plan *plan,
               void *ws, size_t ws_bytes, void *result_host);

// dropzeros: positions of the nonzero entries (count to the host), then the compaction.
size_t dropzeros_workspace_size(int64_t nnz);
template <typename V>
int launch_dropzeros_count(cudaStream_t s, int64_t nnz, const V *val, void *ws, size_t ws_bytes, int64_t *kept);
template <typename V, typename I>
int launch_dropzeros_copy(cudaStream_t s, int fmt, int64_t outer_n, int64_t nnz, const I *p0, const I *p1,
                          const V *val, int base, const void *ws, I *o0, I *o1, V *ov);

// COO sums (A + B, A - B, A + λI): up to two COO sources, each optionally transposed (row
// and column indices swapped), conjugated and negated, then n_diag diagonal entries of value λ.
struct SumSources {
    const void *row[2], *col[2], *val[2];
    int64_t nnz[2], n_diag;
    int trans[2], conj[2], neg[2];
};
size_t coo_sum_workspace_size(size_t vsize, int64_t m, int64_t n, int64_t total);
template <typename V, typename I>
int launch_coo_sum_count(cudaStream_t s, int64_t m, int64_t n, const SumSources &src, const V *lambda, int base,
                         void *ws, size_t ws_bytes, int64_t *kept);
template <typename V, typename I>
int launch_coo_sum_copy(cudaStream_t s, int64_t m, int64_t n, int64_t total, int base, const void *ws, I *row_out,
                        I *col_out, V *val_out);

// C += A for a dense column-major C (fmt 0 CSR, 1 CSC, 2 COO).
template <typename V, typename I>
int launch_add_to_dense(cudaStream_t s, int fmt, int64_t m, int64_t n, int64_t nnz, const I *p0, const I *p1,
                        const V *val, int base, V *C, int64_t ldc);

// COO: out[key_i, c] += conj?(val_i) * (op(B)(other_i, c) * alpha), after the beta pass.
template <typename V, typename I>
int launch_coo(cudaStream_t s, int64_t nnz, const I *out_idx, const I *in_idx, const V *val,
               int base, bool conjA, int64_t k, DenseIn<V> B, DenseOut<V> C, int64_t out_rows,
               int64_t in_rows);

// beta pass of LinearAlgebra._rmul_or_fill! over an out_rows x k block of C.
template <typename V>
int launch_rmul_or_fill(cudaStream_t s, DenseOut<V> C, int64_t out_rows, int64_t k);

// Conversions.
template <typename V, typename I>
int launch_coo_to_compressed(cudaStream_t s, bool colmajor, int64_t m, int64_t n, int64_t nnz,
                             const I *rowind, const I *colind, const V *val, int base,
                             I *ptr_out, I *idx_out, V *val_out, void *ws, size_t ws_bytes);
template <typename V, typename I>
size_t coo_to_compressed_workspace_size(int64_t m, int64_t n, int64_t nnz, bool colmajor);

template <typename I>
int launch_expand_major(cudaStream_t s, int64_t outer_n, int64_t nnz, const I *ptr, int base,
                        I *major_out, void *ws, size_t ws_bytes);
size_t expand_major_workspace_size(int64_t outer_n, int64_t nnz);

template <typename I>
int launch_validate(cudaStream_t s, int64_t outer_n, int64_t inner_n, int64_t nnz, const I *ptr,
                    const I *idx, int base, int *d_flag);

// Merge-path partition shared by gather, scatter and expansion: for each tile
// boundary d = t * tile_items (t = 0..num_tiles), the number of outer entries
// whose end offset is consumed before diagonal d.
template <typename I>
int launch_merge_partition(cudaStream_t s, const I *ptr, int base, int64_t outer_n, int64_t nnz,
                           int64_t tile_items, int64_t num_tiles, int64_t *coords);

}  // namespace gsa
