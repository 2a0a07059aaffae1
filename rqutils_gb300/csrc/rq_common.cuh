// Shared device code of the SQD kernels: value-type traits, compensated accumulation, the
// subspace lookups (hash / sampled binary search / identity), the sector filter and a
// deterministic two-level grid reduction.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rqsqd.h"

namespace rq {

constexpr int kThreads = 256;          // threads per block of the streaming kernels
constexpr int kMaxReduce = 8;          // complex values one grid reduction can carry

// ------------------------------------------------------------------------------------------
// complex values in a given arithmetic precision
// ------------------------------------------------------------------------------------------
template <typename R>
struct cx {
    R re, im;
};

template <typename R>
__device__ __forceinline__ cx<R> cmul(cx<R> a, cx<R> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// Error-free sum (Knuth's TwoSum): s + e == a + b exactly.  Additions only, so FMA contraction
// cannot change it.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Accumulator: compensated (TwoSum with a running error term) in float, plain in double.
template <typename R>
struct Acc;

template <>
struct Acc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        float t, e;
        two_sum(s, v, t, e);
        s = t;
        c += e;
    }
    __device__ __forceinline__ float get() const { return s + c; }
};

template <>
struct Acc<double> {
    double s = 0.;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double get() const { return s; }
};

template <typename R>
struct CAcc {
    Acc<R> re, im;
    __device__ __forceinline__ void add(cx<R> v) {
        re.add(v.re);
        im.add(v.im);
    }
    __device__ __forceinline__ cx<R> get() const { return {re.get(), im.get()}; }
};

// Value-type traits: V is the storage type of a vector element; R the arithmetic precision.
template <typename V>
struct VT;

template <>
struct VT<float> {
    using R = float;
    static constexpr bool kComplex = false;
    static __device__ __forceinline__ cx<float> ld(const float *p, int64_t i) { return {p[i], 0.f}; }
    static __device__ __forceinline__ void st(float *p, int64_t i, cx<float> v) { p[i] = v.re; }
};
template <>
struct VT<double> {
    using R = double;
    static constexpr bool kComplex = false;
    static __device__ __forceinline__ cx<double> ld(const double *p, int64_t i) { return {p[i], 0.}; }
    static __device__ __forceinline__ void st(double *p, int64_t i, cx<double> v) { p[i] = v.re; }
};
template <>
struct VT<float2> {
    using R = float;
    static constexpr bool kComplex = true;
    static __device__ __forceinline__ cx<float> ld(const float2 *p, int64_t i) {
        float2 v = p[i];
        return {v.x, v.y};
    }
    static __device__ __forceinline__ void st(float2 *p, int64_t i, cx<float> v) {
        p[i] = make_float2(v.re, v.im);
    }
};
template <>
struct VT<double2> {
    using R = double;
    static constexpr bool kComplex = true;
    static __device__ __forceinline__ cx<double> ld(const double2 *p, int64_t i) {
        double2 v = p[i];
        return {v.x, v.y};
    }
    static __device__ __forceinline__ void st(double2 *p, int64_t i, cx<double> v) {
        p[i] = make_double2(v.re, v.im);
    }
};

// ------------------------------------------------------------------------------------------
// hashing and lookups
// ------------------------------------------------------------------------------------------
// A bucket holds 4 keys: 16 bytes of uint32 keys when every state and X mask fits in 32 bits,
// else 32 bytes of uint64 keys.  Slots of a bucket fill in order; a full bucket continues the
// probe chain in the next bucket.  The table is sized for a load factor <= 1/8 (half a key per
// bucket on average), so a bucket is full with probability ~0.2% and nearly every lookup is one
// load.
//
// The bucket index comes from a GF(2)-linear hash h(k) = XOR of R[i] over the set bits i of k,
// with fixed pseudo-random 32-bit words R[i].  Linearity gives h(s ^ x) = h(s) ^ h(x): a row
// hashes its state once and each X group contributes one XOR.  h is evaluated with per-byte
// tables T[b][v] = h(v << 8b) kept in shared memory.
__host__ __device__ constexpr uint32_t lin_word(int i) {
    uint32_t h = (uint32_t)(i + 1) * 0x9E3779B9u;
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

constexpr int kHashTableWords = 8 * 256;  // shared-memory words for 64-bit keys
constexpr int kBucketSlots = 4;

// Fill T[b * 256 + v] for b < nbytes (all threads of the block; caller synchronises).
__device__ inline void init_hash_tables(uint32_t *T, int nbytes) {
    for (int idx = threadIdx.x; idx < nbytes * 256; idx += blockDim.x) {
        const int b = idx >> 8, v = idx & 255;
        uint32_t h = 0;
#pragma unroll
        for (int bit = 0; bit < 8; ++bit)
            if ((v >> bit) & 1) h ^= lin_word(8 * b + bit);
        T[idx] = h;
    }
}

__device__ __forceinline__ uint32_t lin_hash(const uint32_t *T, uint64_t k, int nbytes) {
    uint32_t h = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b)
        if (b < nbytes) h ^= T[(b << 8) | (uint32_t)((k >> (8 * b)) & 255u)];
    return h;
}

__device__ __forceinline__ uint32_t bucket_from_hash(uint32_t h, int hbits) {
    return h >> (32 - hbits);
}

// presence bitmap test: bit (h >> (32 - pbits)) of pmap
__device__ __forceinline__ bool present(const uint32_t *pmap, uint32_t h, int pbits) {
    const uint32_t idx = h >> (32 - pbits);
    return (__ldg(pmap + (idx >> 5)) >> (idx & 31)) & 1u;
}

template <int KB>
struct KeyWidth;
template <>
struct KeyWidth<64> {
    using K = uint64_t;
    static constexpr int kNbytes = 8;
    static constexpr int kBucketBytes = 32;
    struct Bucket { uint64_t k[4]; };
    // one 32-byte bucket in a single 256-bit read-only load; `fill` when pred is false
    static __device__ __forceinline__ Bucket load(const void *p, bool pred, uint64_t fill) {
        Bucket b;
        b.k[0] = b.k[1] = b.k[2] = b.k[3] = fill;
        asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %5, 0;\n\t"
            "@q ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];\n\t}"
            : "+l"(b.k[0]), "+l"(b.k[1]), "+l"(b.k[2]), "+l"(b.k[3])
            : "l"(p), "r"((unsigned)pred));
        return b;
    }
};
template <>
struct KeyWidth<32> {
    using K = uint32_t;
    static constexpr int kNbytes = 4;
    static constexpr int kBucketBytes = 16;
    struct Bucket { uint32_t k[4]; };
    static __device__ __forceinline__ Bucket load(const void *p, bool pred, uint64_t fill) {
        Bucket b;
        b.k[0] = b.k[1] = b.k[2] = b.k[3] = (uint32_t)fill;
        asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %5, 0;\n\t"
            "@q ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];\n\t}"
            : "+r"(b.k[0]), "+r"(b.k[1]), "+r"(b.k[2]), "+r"(b.k[3])
            : "l"(p), "r"((unsigned)pred));
        return b;
    }
};

// One 32-bit word of the line filter in a single read-only load; 0 (a miss) when pred is false.
__device__ __forceinline__ uint32_t load_word(const uint32_t *p, bool pred) {
    uint32_t w = 0u;
    asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t"
        "@q ld.global.nc.u32 %0, [%1];\n\t}"
        : "+r"(w)
        : "l"(p), "r"((unsigned)pred));
    return w;
}

// Branch-free bucket test: `any` when a slot equals t, `open` when the last slot is empty.
template <typename Bk, typename K>
__device__ __forceinline__ void test_bucket(const Bk &b, K t, K e, bool &any, bool &open) {
    any = (b.k[0] == t) | (b.k[1] == t) | (b.k[2] == t) | (b.k[3] == t);
    open = (b.k[3] == e);
}

template <typename Bk, typename K>
__device__ __forceinline__ int slot_of(const Bk &b, K t) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (b.k[i] == t) return i;
    return -1;
}

template <int KB>
__device__ __forceinline__ const void *bucket_ptr(const rq_subspace_t &S, uint32_t b) {
    return static_cast<const unsigned char *>(S.hkeys) + (size_t)b * KeyWidth<KB>::kBucketBytes;
}

// Continue a probe chain after a full bucket, bounded by the table size; a chain that never ends
// reports a miss and sets the error flag.
template <int KB>
static __device__ __noinline__ int probe_rest(const rq_subspace_t &S, uint64_t t, uint32_t b,
                                              int *err) {
    using K = typename KeyWidth<KB>::K;
    const uint32_t mask = (1u << S.hbits) - 1u;
    for (uint32_t n = 0; n <= mask; ++n) {
        b = (b + 1) & mask;
        const auto bk = KeyWidth<KB>::load(bucket_ptr<KB>(S, b), true, S.empty_key);
        const int s = slot_of(bk, (K)t);
        if (s >= 0) return S.hvals[(size_t)b * kBucketSlots + s];
        if (bk.k[3] == (K)S.empty_key) return -1;
    }
    if (err) atomicExch(err, RQ_E_TABLE);
    return -1;
}

// Full lookup of t starting at bucket b.  The empty key is not a state, so a target equal to it
// is a miss (it would otherwise match an empty slot, whose row index is undefined).  With 32-bit
// keys every state is below 2^32, so a target at or above it (an X mask with high bits) is a miss
// too: its low 32 bits alone could equal a stored key.
template <int KB>
__device__ __forceinline__ int lookup_hash_at(const rq_subspace_t &S, uint64_t t, uint32_t b,
                                              int *err) {
    using K = typename KeyWidth<KB>::K;
    if (t == S.empty_key || (KB == 32 && (t >> 32) != 0)) return -1;
    // the bucket's four row indices load beside its keys (independent addresses; hvals is 16-byte
    // aligned), so a hit costs one round trip to the table instead of two
    const int4 v = __ldg(reinterpret_cast<const int4 *>(S.hvals) + b);
    const auto bk = KeyWidth<KB>::load(bucket_ptr<KB>(S, b), true, S.empty_key);
    const int s = slot_of(bk, (K)t);
    if (s >= 0) return s == 0 ? v.x : s == 1 ? v.y : s == 2 ? v.z : v.w;
    if (bk.k[3] == (K)S.empty_key) return -1;
    return probe_rest<KB>(S, t, b, err);
}

// Sampled binary search: `samp` (shared memory) holds states[(k * D) / ns] for k < ns.  The
// sample narrows the range to at most ceil(D / ns) + 1 entries, searched in global memory.
__device__ __forceinline__ int lookup_bsearch(const rq_subspace_t &S, const uint64_t *samp,
                                              int ns, uint64_t t) {
    const int64_t D = S.D;
    int lo = 0, hi = ns;  // largest k with samp[k] <= t
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (samp[mid] <= t) lo = mid; else hi = mid;
    }
    if (samp[lo] > t) return -1;
    int64_t a = ((int64_t)lo * D) / ns;
    int64_t b = (lo + 1 < ns) ? ((int64_t)(lo + 1) * D) / ns : D;  // exclusive
    while (b - a > 1) {
        int64_t mid = (a + b) >> 1;
        if (__ldg(S.states + mid) <= t) a = mid; else b = mid;
    }
    return (__ldg(S.states + a) == t) ? (int)a : -1;
}

// Sector filter: bit (popcount(t & a) * 65 + popcount(t & b)) of the 65 x 65 table.
__device__ __forceinline__ bool sector_ok(const uint32_t *fb, uint64_t a, uint64_t b, uint64_t t) {
    const int bit = __popcll(t & a) * 65 + __popcll(t & b);
    return (fb[bit >> 5] >> (bit & 31)) & 1u;
}

template <typename K>
__device__ __forceinline__ bool sector_ok_k(const uint32_t *fb, K a, K b, K t) {
    int pa, pb;
    if (sizeof(K) == 8) {
        pa = __popcll((unsigned long long)(t & a));
        pb = __popcll((unsigned long long)(t & b));
    } else {
        pa = __popc((unsigned)(t & a));
        pb = __popc((unsigned)(t & b));
    }
    const int bit = pa * 65 + pb;
    return (fb[bit >> 5] >> (bit & 31)) & 1u;
}

// ------------------------------------------------------------------------------------------
// double-float sums: GB300 issues FP64 at a small fraction of its FP32 rate, so reduction trees
// (shuffles, shared memory, the last block's pass over the partials) add pairs of floats
// (hi + lo, ~48-bit significand) instead of doubles
// ------------------------------------------------------------------------------------------
struct df {
    float hi, lo;
};
struct cdf {
    df re, im;
};

__device__ __forceinline__ df df_of(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_val(df a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df df_add(df a, df b) {
    float s, e, t, f;
    two_sum(a.hi, b.hi, s, e);
    two_sum(a.lo, b.lo, t, f);
    e += t;
    float h = s + e;
    e = e - (h - s);
    e += f;
    s = h + e;
    e = e - (s - h);
    return {s, e};
}
__device__ __forceinline__ cdf cdf_add(cdf a, cdf b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ double2 cdf_val(cdf a) { return make_double2(df_val(a.re), df_val(a.im)); }
__device__ __forceinline__ cdf cdf_shfl_xor(cdf a, int o) {
    return {{__shfl_xor_sync(0xffffffffu, a.re.hi, o), __shfl_xor_sync(0xffffffffu, a.re.lo, o)},
            {__shfl_xor_sync(0xffffffffu, a.im.hi, o), __shfl_xor_sync(0xffffffffu, a.im.lo, o)}};
}
__device__ __forceinline__ cdf cdf_zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
__device__ __forceinline__ float4 cdf_pack(cdf a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ cdf cdf_unpack(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }

// Block-wide sums of NV <= 8 values, left in tot[0..NV) (shared memory) for every thread.
// Within a warp the values are reduce-scattered: at each of the first log2(P) butterfly steps
// (P = NV rounded up to a power of two) a lane keeps half of its values and receives the
// partner's partial sums of that half, so a lane adds P - 1 + (5 - log2 P) pairs instead of
// 5 NV; afterwards the lanes of one value hold its warp total.  Across warps, warp k sums
// value k.  The order of every addition is fixed, so each block computes the same sums from
// the same inputs.
template <int NV>
__device__ __forceinline__ void block_sum_all(cdf (&w)[NV], cdf *tot, cdf (*red)[NV]) {
    static_assert(NV >= 1 && NV <= 8, "block_sum_all: at most 8 values");
    constexpr int L = NV <= 1 ? 0 : NV <= 2 ? 1 : NV <= 4 ? 2 : 3;  // halving steps
    constexpr int P = 1 << L;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
    cdf a[P];
#pragma unroll
    for (int k = 0; k < P; ++k) a[k] = k < NV ? w[k] : cdf_zero();
#pragma unroll
    for (int s = 0; s < L; ++s) {
        const int o = 16 >> s, h = P >> (s + 1);
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const cdf mine = up ? a[h + j] : a[j];
            const cdf other = up ? a[j] : a[h + j];
            a[j] = cdf_add(mine, cdf_shfl_xor(other, o));
        }
    }
#pragma unroll
    for (int s = L; s < 5; ++s) a[0] = cdf_add(a[0], cdf_shfl_xor(a[0], 16 >> s));
    int v = 0;
#pragma unroll
    for (int s = 0; s < L; ++s) v += ((lane >> (4 - s)) & 1) * (P >> (s + 1));
    if ((lane & ((32 >> L) - 1)) == 0 && v < NV) red[warp][v] = a[0];
    __syncthreads();
    for (int k = warp; k < NV; k += nwarp) {
        cdf t = lane < nwarp ? red[lane][k] : cdf_zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = cdf_add(t, cdf_shfl_xor(t, o));
        if (lane == 0) tot[k] = t;
    }
    __syncthreads();
}

// Sums of NV values over n per-block partials (float4-packed double-floats, stride `stride`),
// warp k summing value k; left in tot[0..NV) for every thread.
template <int NV>
__device__ __forceinline__ void partials_sum(const float4 *part, int n, int stride, cdf *tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
    for (int k = warp; k < NV; k += nwarp) {
        cdf t = cdf_zero();
#pragma unroll 4
        for (int b = lane; b < n; b += 32) t = cdf_add(t, cdf_unpack(__ldcg(part + (size_t)b * stride + k)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t = cdf_add(t, cdf_shfl_xor(t, o));
        if (lane == 0) tot[k] = t;
    }
    __syncthreads();
}

// ------------------------------------------------------------------------------------------
// deterministic grid reduction of NV complex values
// ------------------------------------------------------------------------------------------
// Scratch layout: [counter (uint32, 16 B slot)] [partials: gridDim.x * NV double-float pairs].
// Each block writes its partials; the last block to finish sums them in block order and writes
// `out`, then resets the counter so the scratch can be reused by the next launch.
template <int NV>
__device__ void grid_reduce(cdf (&v)[NV], void *scratch, double2 *out) {
    __shared__ cdf red[kThreads / 32][NV];
    __shared__ cdf tot[NV];
    __shared__ bool last;
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch);
    float4 *part = reinterpret_cast<float4 *>(reinterpret_cast<char *>(scratch) + 16);
    cdf w[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) w[k] = v[k];
    block_sum_all<NV>(w, tot, red);
    if (threadIdx.x < NV) {
        part[(size_t)blockIdx.x * NV + threadIdx.x] = cdf_pack(tot[threadIdx.x]);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    partials_sum<NV>(part, (int)gridDim.x, NV, tot);
    if (threadIdx.x < NV) out[threadIdx.x] = cdf_val(tot[threadIdx.x]);
    if (threadIdx.x == 0) *counter = 0u;
}

// Max blocks a reducing launch may use (sizes the partials of the scratch area).
constexpr int kMaxReduceBlocks = 4096;

inline size_t reduce_scratch_bytes() {
    return 16 + (size_t)kMaxReduceBlocks * kMaxReduce * sizeof(double2);
}

}  // namespace rq
