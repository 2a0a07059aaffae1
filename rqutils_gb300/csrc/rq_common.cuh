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
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t k) {
    k ^= k >> 31;
    k *= 0x7fb5d329728ea185ULL;
    k ^= k >> 27;
    k *= 0x81dadef4bc2dd44dULL;
    k ^= k >> 33;
    return k;
}

__device__ __forceinline__ uint64_t bucket_of(uint64_t key, int hbits) {
    return mix64(key) >> (64 - hbits);
}

// One 32-byte bucket (4 keys) in a single 256-bit read-only load.
__device__ __forceinline__ void load_bucket(const uint64_t *p, uint64_t &k0, uint64_t &k1,
                                            uint64_t &k2, uint64_t &k3) {
    asm volatile("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];"
                 : "=l"(k0), "=l"(k1), "=l"(k2), "=l"(k3)
                 : "l"(p));
}

// Slot of `t` among the four keys, -1 when absent; `open` is set when the bucket still has an
// empty slot (slots fill in order, so an empty last slot ends the probe chain).
__device__ __forceinline__ int match_bucket(uint64_t t, uint64_t empty, uint64_t k0, uint64_t k1,
                                            uint64_t k2, uint64_t k3, bool &open) {
    open = (k3 == empty);
    if (k0 == t) return 0;
    if (k1 == t) return 1;
    if (k2 == t) return 2;
    if (k3 == t) return 3;
    return -1;
}

// Continue a probe chain after a full bucket (rare at load factor <= 1/2).  Bounded by the
// table size; a chain that never ends reports a miss and sets the error flag.
static __device__ __noinline__ int probe_rest(const rq_subspace_t &S, uint64_t t, uint64_t b,
                                       int *err) {
    const uint64_t mask = (1ULL << S.hbits) - 1;
    for (uint64_t n = 0; n <= mask; ++n) {
        b = (b + 1) & mask;
        uint64_t k0, k1, k2, k3;
        load_bucket(S.hkeys + (b << 2), k0, k1, k2, k3);
        bool open;
        int s = match_bucket(t, S.empty_key, k0, k1, k2, k3, open);
        if (s >= 0) return S.hvals[(b << 2) + s];
        if (open) return -1;
    }
    if (err) atomicExch(err, RQ_E_TABLE);
    return -1;
}

// The empty key is not a state, so a target equal to it is a miss (it would otherwise match an
// empty slot, whose row index is undefined).
__device__ __forceinline__ int lookup_hash(const rq_subspace_t &S, uint64_t t, int *err) {
    if (t == S.empty_key) return -1;
    const uint64_t b = bucket_of(t, S.hbits);
    uint64_t k0, k1, k2, k3;
    load_bucket(S.hkeys + (b << 2), k0, k1, k2, k3);
    bool open;
    int s = match_bucket(t, S.empty_key, k0, k1, k2, k3, open);
    if (s >= 0) return S.hvals[(b << 2) + s];
    if (open) return -1;
    return probe_rest(S, t, b, err);
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

// ------------------------------------------------------------------------------------------
// deterministic grid reduction of NV complex doubles
// ------------------------------------------------------------------------------------------
// Scratch layout: [counter (uint32, 16 B slot)] [partials: gridDim.x * NV double2].
// Each block writes its partials; the last block to finish sums them in block order and writes
// `out`, then resets the counter so the scratch can be reused by the next launch.
template <int NV>
__device__ void grid_reduce(double2 (&v)[NV], void *scratch, double2 *out) {
    __shared__ double2 red[kThreads / 32][NV];
    __shared__ bool last;
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch);
    double2 *part = reinterpret_cast<double2 *>(reinterpret_cast<char *>(scratch) + 16);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarp = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v[k].x += __shfl_xor_sync(0xffffffffu, v[k].x, o);
            v[k].y += __shfl_xor_sync(0xffffffffu, v[k].y, o);
        }
        if (lane == 0) red[warp][k] = v[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double2 a = (lane < nwarp) ? red[lane][k] : make_double2(0., 0.);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
                a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
            }
            if (lane == 0) part[(size_t)blockIdx.x * NV + k] = a;
        }
        if (lane == 0) {
            __threadfence();
            unsigned int t = atomicAdd(counter, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double2 a = make_double2(0., 0.);
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
            double2 p = __ldcg(part + (size_t)b * NV + k);
            a.x += p.x;
            a.y += p.y;
        }
        v[k] = a;
    }
    __syncthreads();  // red[] reuse
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v[k].x += __shfl_xor_sync(0xffffffffu, v[k].x, o);
            v[k].y += __shfl_xor_sync(0xffffffffu, v[k].y, o);
        }
        if (lane == 0) red[warp][k] = v[k];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double2 a = (lane < nwarp) ? red[lane][k] : make_double2(0., 0.);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
                a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
            }
            if (lane == 0) out[k] = a;
        }
        if (lane == 0) *counter = 0u;
    }
}

// Max blocks a reducing launch may use (sizes the partials of the scratch area).
constexpr int kMaxReduceBlocks = 4096;

inline size_t reduce_scratch_bytes() {
    return 16 + (size_t)kMaxReduceBlocks * kMaxReduce * sizeof(double2);
}

}  // namespace rq
