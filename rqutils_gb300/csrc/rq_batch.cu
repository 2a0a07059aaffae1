// Batches of independent SQD problems on one device.
//
// Every problem's states are stored as composite keys (p << 40) | s, sorted, in one array, and
// one hash table holds them all.  The lookup hash is GF(2)-linear, so the bucket of a target
// (p << 40) | (s ^ x) is h(row key) ^ h(x): the probe loop of a row is the single-problem one,
// only the row's group range, x = 0 group and sector filter come from its problem.
#include <string>
#include <vector>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {

int build_key_table(const uint64_t *keys, int64_t D, int key_bits, bool hash, void *hkeys,
                    int32_t *hvals, int hbits, uint64_t *empty_out, int *flag,
                    unsigned long long *gap, cudaStream_t st, uint32_t *pmap, int pbits);

namespace {

constexpr int kStateBits = RQ_BATCH_STATE_BITS;
constexpr uint64_t kStateMask = (1ULL << kStateBits) - 1ULL;

__device__ __forceinline__ int problem_of(uint64_t key) { return (int)(key >> kStateBits); }

int grid_rows(int64_t n, int per_sm = 8) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

// every row's problem id must match the row ranges (keys of problem p between prow[p], prow[p+1])
__global__ void k_batch_check_rows(const uint64_t *__restrict__ keys, int64_t D,
                                   const int64_t *__restrict__ prow, int P, int *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int p = problem_of(keys[i]);
        if (p >= P || i < prow[p] || i >= prow[p + 1]) atomicExch(flag, 1);
    }
}

// X masks must stay inside the state bits (a flip of a problem bit would reach another problem)
__global__ void k_batch_check_terms(const uint64_t *__restrict__ xmask, int J, int *flag) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < J; g += gridDim.x * blockDim.x)
        if (xmask[g] & ~kStateMask) atomicExch(flag, 2);
}

// per-problem sector filter bits; a word is written only when its bit is missing
__global__ void k_batch_filters(const uint64_t *__restrict__ keys, int64_t D,
                                const uint64_t *__restrict__ fmask, uint32_t *fbits) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const int p = problem_of(k);
        const uint64_t s = k & kStateMask;
        const int bit = __popcll(s & fmask[2 * p]) * 65 + __popcll(s & fmask[2 * p + 1]);
        uint32_t *w = fbits + (size_t)p * RQ_FILTER_WORDS + (bit >> 5);
        const uint32_t m = 1u << (bit & 31);
        if (!(*(volatile uint32_t *)w & m)) atomicOr(w, m);
    }
}

__global__ void k_fill_all_bits(uint32_t *fbits, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        fbits[i] = 0xFFFFFFFFu;
}

// x = 0 diagonal of each row from its problem's diagonal group (FP64, stop at the first zero)
__global__ void k_batch_diag(const uint64_t *__restrict__ keys, int64_t D, const int32_t *__restrict__ dgrp,
                             const rq_terms_t T, double *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const int g = dgrp[problem_of(k)];
        const uint64_t s = k & kStateMask;
        double d = 0.;
        if (g >= 0) {
            const int k1 = __ldg(T.toff + g + 1);
            for (int t = __ldg(T.toff + g); t < k1; ++t) {
                const double c = __ldg(T.coef + 2 * t);
                if (c == 0. && __ldg(T.coef + 2 * t + 1) == 0.) break;
                d += (__popcll(s & __ldg(T.zmask + t)) & 1) ? -c : c;
            }
        }
        out[i] = d;
    }
}

template <typename R>
__device__ __forceinline__ cx<R> bgroup_diag(const rq_terms_t &T, int g, uint64_t s) {
    CAcc<R> d;
    const int k1 = __ldg(T.toff + g + 1);
    for (int k = __ldg(T.toff + g); k < k1; ++k) {
        const R re = (R)__ldg(T.coef + 2 * k), im = (R)__ldg(T.coef + 2 * k + 1);
        if (re == (R)0 && im == (R)0) break;
        if (__popcll(s & __ldg(T.zmask + k)) & 1) d.add({-re, -im});
        else d.add({re, im});
    }
    return d.get();
}

// Line filter of a batch, per problem p (block p): the prefix shift lshift[p] from the highest
// differing bit of the problem's neighbouring keys (the largest shift with about 2^(lwbits - 5)
// keys per distinct prefix, as for one subspace), then xline[g] = hash(xmask[g] >> lshift[p]) for
// the problem's groups.
__global__ void __launch_bounds__(kThreads)
k_batch_line_prep(const uint64_t *__restrict__ keys, const int64_t *__restrict__ prow,
                  const uint64_t *__restrict__ xmask, const int32_t *__restrict__ gofs, int lwbits,
                  int32_t *__restrict__ lshift, uint32_t *__restrict__ xline) {
    __shared__ uint32_t T[kHashTableWords];
    __shared__ unsigned int hist[64];
    __shared__ int shift_s;
    const int p = blockIdx.x;
    init_hash_tables(T, 8);
    if (threadIdx.x < 64) hist[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t r0 = prow[p], r1 = prow[p + 1];
    for (int64_t i = r0 + 1 + threadIdx.x; i < r1; i += blockDim.x)
        atomicAdd(&hist[63 - __clzll((long long)(keys[i] ^ keys[i - 1]))], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        const double per = (double)(1 << (lwbits - 5));
        const double Dp = (double)(r1 - r0);
        unsigned long long above = 0;  // distinct prefixes at shift b, minus one
        for (int k = 0; k < 64; ++k) above += hist[k];
        int b = 0;
        for (int c = 1; c <= kStateBits; ++c) {
            above -= hist[c - 1];
            if (Dp > per * (double)(above + 1)) break;
            b = c;
        }
        shift_s = b;
        lshift[p] = b;
    }
    __syncthreads();
    const int b = shift_s;
    for (int g = gofs[p] + threadIdx.x; g < gofs[p + 1]; g += blockDim.x) xline[g] = lin_hash(T, xmask[g] >> b, 8);
}

// for every key (h = hash(key)): bits h mod 32 and h >> 27 of word (h mod 2^lwbits) >> 5 of line
// hash(key >> lshift[p]) >> (32 - lbits)
__global__ void __launch_bounds__(kThreads)
k_batch_line_build(const uint64_t *__restrict__ keys, int64_t D, const int32_t *__restrict__ lshift,
                   uint32_t *__restrict__ lmap, int lbits, int lwbits) {
    __shared__ uint32_t T[kHashTableWords];
    init_hash_tables(T, 8);
    __syncthreads();
    const uint32_t bmask = (1u << lwbits) - 1u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        const uint32_t line = lin_hash(T, k >> lshift[problem_of(k)], 8) >> (32 - lbits);
        const uint32_t h = lin_hash(T, k, 8);
        atomicOr(lmap + ((size_t)line << (lwbits - 5)) + ((h & bmask) >> 5), (1u << (h & 31)) | (1u << (h >> 27)));
    }
}

__device__ __forceinline__ bool gate_open(const int *gate, int64_t stride, const int *gate2, int p) {
    if (!gate) return true;
    if (!*reinterpret_cast<const int *>(reinterpret_cast<const char *>(gate) + p * stride))
        return false;
    return !gate2 || *reinterpret_cast<const int *>(reinterpret_cast<const char *>(gate2) + p * stride);
}

// Visit the hits of one row (warp-uniform group loop so the warp can re-converge after each
// 64-group resolution): on_hit(g, m).  `act` rows probe; inactive lanes run the loop empty.
// Per chunk of 64 groups the sector filter runs first and leaves a mask of the groups whose
// target can be in the problem's sector; the bucket probes then walk only those groups, U at a
// time per lane (random Pauli sums keep about one target in five in the sector, so most of the
// probe work of a chunk is never issued).
template <typename F>
__device__ __forceinline__ void batch_row_hits(const rq_batch_t &B, const uint32_t *htab, bool act,
                                               uint64_t key, int *err, F &&on_hit) {
    const int p = act ? problem_of(key) : 0;
    const int g0 = act ? B.gofs[p] : 0;
    const int ng = act ? B.gofs[p + 1] - g0 : 0;
    const int skip = act ? B.dgrp[p] - g0 : -1;
    const int nmax = __reduce_max_sync(0xffffffffu, ng);
    const uint64_t fa = (act && B.fmask) ? B.fmask[2 * p] : 0ULL;
    const uint64_t fbm = (act && B.fmask) ? B.fmask[2 * p + 1] : 0ULL;
    const uint32_t *fb = B.fbits + (size_t)p * RQ_FILTER_WORDS;
    const uint64_t s = key & kStateMask;
    const uint32_t hs = lin_hash(htab, key, 8);
    const int shift = 32 - B.hbits;
    const rq_subspace_t S = {nullptr, B.D, B.hkeys, B.hvals, B.hbits, RQ_LOOKUP_HASH, 64, 0,
                             B.empty_key, 0, 0, nullptr};
    const unsigned char *keys = static_cast<const unsigned char *>(B.hkeys);
    const uint64_t *xm = B.terms.xmask + g0;
    const uint32_t *xh = B.terms.xhash + g0;
    const uint32_t *xl = B.lmap ? B.xline + g0 : nullptr;
    // line filter: the row's prefix hash once; a target's line is (hls ^ xline[g]) >> lsh
    const uint32_t hls = (B.lmap && act) ? lin_hash(htab, key >> B.lshift[p], 8) : 0u;
    const int lsh = 32 - B.lbits, lwsh = B.lwbits - 5;
    const uint32_t lbmask = (1u << B.lwbits) - 1u;
    constexpr int U = 4;
    for (int r0 = 0; r0 < nmax; r0 += 64) {
        const int r1 = min(ng, r0 + 64);
        // groups of the chunk whose target passes the sector filter, four at a time so that
        // their X-mask and filter-word loads overlap
        uint64_t pass = 0ULL;
        for (int r = r0; r < r1; r += 4) {
            uint64_t xv[4];
            int bit[4];
            uint32_t fw[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) xv[u] = r + u < r1 ? __ldg(xm + r + u) : 0ULL;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint64_t ts = s ^ xv[u];
                bit[u] = __popcll(ts & fa) * 65 + __popcll(ts & fbm);
                fw[u] = (r + u < r1 && B.fmask) ? __ldg(fb + (bit[u] >> 5)) : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = r + u < r1 && r + u != skip && (key ^ xv[u]) != B.empty_key &&
                                ((fw[u] >> (bit[u] & 31)) & 1u);
                if (ok) pass |= 1ULL << (r + u - r0);
            }
        }
        uint64_t hot = 0ULL;
        if (xl) {
            // line filter: a group whose target sets both bits is resolved below (the lookup
            // reads its bucket), so only filter words are in flight, eight per thread
            constexpr int UL = 8;
            while (__any_sync(0xffffffffu, pass != 0ULL)) {
                int rr[UL];
                uint32_t b[UL], lw[UL];
                bool q[UL];
#pragma unroll
                for (int u = 0; u < UL; ++u) {
                    q[u] = pass != 0ULL;
                    rr[u] = q[u] ? __ffsll((long long)pass) - 1 : 0;
                    pass &= pass - 1ULL;
                    b[u] = hs ^ (q[u] ? __ldg(xh + r0 + rr[u]) : 0u);
                    const uint32_t ln = q[u] ? (hls ^ __ldg(xl + r0 + rr[u])) >> lsh : 0u;
                    lw[u] = q[u] ? __ldg(B.lmap + ((size_t)ln << lwsh) + ((b[u] & lbmask) >> 5)) : 0u;
                }
#pragma unroll
                for (int u = 0; u < UL; ++u)
                    if (q[u] && ((lw[u] >> (b[u] & 31)) & (lw[u] >> (b[u] >> 27)) & 1u)) hot |= 1ULL << rr[u];
            }
        } else {
            while (__any_sync(0xffffffffu, pass != 0ULL)) {
                int rr[U];
                uint64_t t[U];
                uint32_t b[U];
                bool q[U];
                typename KeyWidth<64>::Bucket w[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    q[u] = pass != 0ULL;
                    rr[u] = q[u] ? __ffsll((long long)pass) - 1 : 0;
                    pass &= pass - 1ULL;
                    const uint64_t xv = q[u] ? __ldg(xm + r0 + rr[u]) : 0ULL;
                    const uint32_t hx = q[u] ? __ldg(xh + r0 + rr[u]) : 0u;
                    t[u] = key ^ xv;
                    b[u] = hs ^ hx;
                }
                if (B.pbits > 0) {
                    uint32_t pw[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const uint32_t idx = b[u] >> (32 - B.pbits);
                        pw[u] = q[u] ? __ldg(B.pmap + (idx >> 5)) : 0u;
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        q[u] = q[u] && ((pw[u] >> ((b[u] >> (32 - B.pbits)) & 31)) & 1u);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
                    w[u] = KeyWidth<64>::load(keys + (size_t)(b[u] >> shift) * 32, q[u], B.empty_key);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    bool any, open;
                    test_bucket(w[u], t[u], B.empty_key, any, open);
                    if (q[u] && (any || !open)) hot |= 1ULL << rr[u];
                }
            }
        }
        while (hot) {
            const int r = r0 + __ffsll((long long)hot) - 1;
            hot &= hot - 1ULL;
            const int m = lookup_hash_at<64>(S, key ^ __ldg(xm + r), (hs ^ __ldg(xh + r)) >> shift, err);
            if (m >= 0) on_hit(g0 + r, m);
        }
        __syncwarp();
    }
}

// FREE-mode batched matvec: thread per row.
template <typename V>
__global__ void __launch_bounds__(kThreads, 4)
k_batch_matvec_free(const rq_batch_t B, const V *__restrict__ x, V *__restrict__ y, int *err,
                    const int *gate, int64_t gstride, const int *gate2) {
    using R = typename VT<V>::R;
    __shared__ uint32_t htab[kHashTableWords];
    init_hash_tables(htab, 8);
    __syncthreads();
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < B.D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        bool act = i < B.D;
        const uint64_t key = act ? __ldg(B.keys + i) : 0ULL;
        act = act && gate_open(gate, gstride, gate2, problem_of(key));
        CAcc<R> acc;
        if (act) {
            const cx<R> xi = VT<V>::ld(x, i);
            const R dv = (R)B.diag0[i];
            acc.add({dv * xi.re, dv * xi.im});
        }
        const uint64_t s = key & kStateMask;
        batch_row_hits(B, htab, act, key, err, [&](int g, int m) {
            acc.add(cmul(bgroup_diag<R>(B.terms, g, s), VT<V>::ld(x, m)));
        });
        if (act) VT<V>::st(y, i, acc.get());
    }
}

__global__ void __launch_bounds__(kThreads)
k_batch_conn_count(const rq_batch_t B, int64_t *__restrict__ rowcnt, int *err) {
    __shared__ uint32_t htab[kHashTableWords];
    init_hash_tables(htab, 8);
    __syncthreads();
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < B.D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const bool act = i < B.D;
        const uint64_t key = act ? __ldg(B.keys + i) : 0ULL;
        int64_t c = 0;
        batch_row_hits(B, htab, act, key, err, [&](int, int) { ++c; });
        if (act) rowcnt[i] = c;
    }
}

__global__ void __launch_bounds__(kThreads)
k_batch_conn_fill(const rq_batch_t B, const int64_t *__restrict__ rowptr, int32_t *__restrict__ col,
                  int32_t *__restrict__ grp, int *err) {
    __shared__ uint32_t htab[kHashTableWords];
    init_hash_tables(htab, 8);
    __syncthreads();
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < B.D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const bool act = i < B.D;
        const uint64_t key = act ? __ldg(B.keys + i) : 0ULL;
        int64_t p = act ? rowptr[i] : 0;
        batch_row_hits(B, htab, act, key, err, [&](int g, int m) {
            col[p] = m;
            grp[p] = g;
            ++p;
        });
    }
}

template <typename V>
__global__ void __launch_bounds__(kThreads)
k_batch_matvec_conn(const rq_batch_t B, const V *__restrict__ x, V *__restrict__ y,
                    const int *gate, int64_t gstride, const int *gate2) {
    using R = typename VT<V>::R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B.D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = __ldg(B.keys + i);
        if (!gate_open(gate, gstride, gate2, problem_of(key))) continue;
        const uint64_t s = key & kStateMask;
        CAcc<R> acc;
        const cx<R> xi = VT<V>::ld(x, i);
        const R dv = (R)B.diag0[i];
        acc.add({dv * xi.re, dv * xi.im});
        const int64_t e1 = B.rowptr[i + 1];
        for (int64_t e = B.rowptr[i]; e < e1; ++e)
            acc.add(cmul(bgroup_diag<R>(B.terms, __ldg(B.grp + e), s),
                         VT<V>::ld(x, __ldg(B.col + e))));
        VT<V>::st(y, i, acc.get());
    }
}

// scans of the CONN build live in rq_matvec.cu
}  // namespace

int scan_row_counts(int64_t *rowptr_plus1, int64_t D, int64_t *bsum, cudaStream_t st);

template <typename V>
int batch_matvec_typed(const rq_batch_t &B, const void *x, void *y, int *err, cudaStream_t st,
                       const int *gate, int64_t gstride, const int *gate2) {
    if (B.mode == RQ_MODE_FREE) {
        k_batch_matvec_free<V><<<grid_rows(B.D, 6), kThreads, 0, st>>>(
            B, static_cast<const V *>(x), static_cast<V *>(y), err, gate, gstride, gate2);
    } else if (B.mode == RQ_MODE_CONN) {
        if (!B.rowptr || (B.nnz > 0 && (!B.col || !B.grp)))
            return fail(RQ_E_ARG, "rq_batch_matvec: RQ_MODE_CONN needs rowptr, col and grp");
        k_batch_matvec_conn<V><<<grid_rows(B.D), kThreads, 0, st>>>(
            B, static_cast<const V *>(x), static_cast<V *>(y), gate, gstride, gate2);
    } else {
        return fail(RQ_E_ARG, "rq_batch_matvec: mode must be RQ_MODE_FREE or RQ_MODE_CONN");
    }
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

int batch_matvec_dispatch(const rq_batch_t &B, int32_t vt, const void *x, void *y, void *scratch,
                          cudaStream_t st, const int *gate, int64_t gstride, const int *gate2) {
    int *err = scratch ? scratch_err(scratch) : nullptr;
    switch (vt) {
        case RQ_F32: return batch_matvec_typed<float>(B, x, y, err, st, gate, gstride, gate2);
        case RQ_F64: return batch_matvec_typed<double>(B, x, y, err, st, gate, gstride, gate2);
        case RQ_C64: return batch_matvec_typed<float2>(B, x, y, err, st, gate, gstride, gate2);
        case RQ_C128: return batch_matvec_typed<double2>(B, x, y, err, st, gate, gstride, gate2);
        default: return fail(RQ_E_ARG, "unknown value type");
    }
}

int check_batch(const rq_batch_t *b) {
    if (!b || !b->keys || !b->prow || !b->gofs || !b->dgrp || !b->diag0 || !b->fbits)
        return fail(RQ_E_ARG, "rq_batch: null array");
    if (b->P < 1 || b->P >= (1 << (64 - kStateBits)))
        return fail(RQ_E_RANGE, "rq_batch: P out of range");
    if (b->D < 1 || b->D >= (int64_t(1) << 31)) return fail(RQ_E_RANGE, "rq_batch: D out of range");
    const rq_terms_t &T = b->terms;
    if (T.J < 0 || (T.J > 0 && (!T.xmask || !T.toff || !T.xhash)) ||
        (T.K > 0 && (!T.zmask || !T.coef)))
        return fail(RQ_E_ARG, "rq_batch: terms need xmask, toff, zmask, coef and xhash");
    if (!b->hkeys || !b->hvals || b->hbits < 1 || b->hbits > 31)
        return fail(RQ_E_ARG, "rq_batch: hash buffers missing or hbits out of range");
    return RQ_OK;
}

}  // namespace rq

using namespace rq;

RQ_API int rq_batch_build(rq_batch_t *b, void *scratch, void *stream) {
    RQ_TRY(check_batch(b));
    if (!scratch) return fail(RQ_E_ARG, "rq_batch_build: null scratch");
    if ((int64_t(kBucketSlots) << b->hbits) < b->D + 1)
        return fail(RQ_E_ARG, "rq_batch_build: hash table too small");
    cudaStream_t st = as_stream(stream);
    {   // group ranges: gofs nondecreasing over [0, J], dgrp inside its problem's range or -1
        std::vector<int32_t> gofs(b->P + 1), dgrp(b->P);
        RQ_CUDA(cudaMemcpyAsync(gofs.data(), b->gofs, sizeof(int32_t) * (b->P + 1),
                                cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaMemcpyAsync(dgrp.data(), b->dgrp, sizeof(int32_t) * b->P,
                                cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        if (gofs[0] != 0 || gofs[b->P] != b->terms.J)
            return fail(RQ_E_ARG, "rq_batch_build: gofs must span [0, J]");
        for (int p = 0; p < b->P; ++p)
            if (gofs[p + 1] < gofs[p] || (dgrp[p] != -1 && (dgrp[p] < gofs[p] || dgrp[p] >= gofs[p + 1])))
                return fail(RQ_E_ARG, "rq_batch_build: bad gofs / dgrp of a problem");
    }
    int *flag = scratch_err(scratch);
    unsigned long long *gap = reinterpret_cast<unsigned long long *>(scratch);
    if (b->pbits != 0 && (!b->pmap || b->pbits < 5 || b->pbits > 32 || b->pbits < b->hbits))
        return fail(RQ_E_ARG, "rq_batch_build: presence bitmap missing or pbits out of range");
    if (b->lmap && (!b->xline || !b->lshift || b->lbits < 1 || b->lbits > 31 || b->lwbits < 8 || b->lwbits > 10))
        return fail(RQ_E_ARG, "rq_batch_build: line filter needs xline, lshift, 1 <= lbits <= 31, 8 <= lwbits <= 10");
    int rc = build_key_table(b->keys, b->D, 64, true, b->hkeys, b->hvals, b->hbits, &b->empty_key,
                             flag, gap, st, b->pbits ? b->pmap : nullptr, b->pbits);
    if (rc != RQ_OK) return fail(rc, std::string("rq_batch_build: ") + rq_last_error());
    RQ_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    k_batch_check_rows<<<grid_rows(b->D), kThreads, 0, st>>>(b->keys, b->D, b->prow, b->P, flag);
    if (b->terms.J > 0)
        k_batch_check_terms<<<grid_rows(b->terms.J), kThreads, 0, st>>>(b->terms.xmask,
                                                                       b->terms.J, flag);
    const int64_t nwords = (int64_t)b->P * RQ_FILTER_WORDS;
    if (b->fmask) {
        RQ_CUDA(cudaMemsetAsync(b->fbits, 0, nwords * sizeof(uint32_t), st));
        k_batch_filters<<<grid_rows(b->D), kThreads, 0, st>>>(b->keys, b->D, b->fmask, b->fbits);
    } else {
        k_fill_all_bits<<<grid_rows(nwords), kThreads, 0, st>>>(b->fbits, nwords);
    }
    k_batch_diag<<<grid_rows(b->D), kThreads, 0, st>>>(b->keys, b->D, b->dgrp, b->terms, b->diag0);
    if (b->lmap) {
        k_batch_line_prep<<<b->P, kThreads, 0, st>>>(b->keys, b->prow, b->terms.xmask, b->gofs, b->lwbits,
                                                      b->lshift, b->xline);
        RQ_CUDA(cudaMemsetAsync(b->lmap, 0, (size_t)1 << (b->lbits + b->lwbits - 3), st));
        k_batch_line_build<<<grid_rows(b->D), kThreads, 0, st>>>(b->keys, b->D, b->lshift, b->lmap, b->lbits,
                                                                  b->lwbits);
    }
    RQ_CUDA(cudaGetLastError());
    int h_flag = 0;
    RQ_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    if (h_flag == 2) return fail(RQ_E_RANGE, "rq_batch_build: an X mask has bits above the state bits");
    if (h_flag) return fail(RQ_E_ARG, "rq_batch_build: keys do not match the problem row ranges");
    return RQ_OK;
}

RQ_API int rq_batch_conn_build(const rq_batch_t *b, int64_t *rowptr, int32_t *col, int32_t *grp,
                               int64_t *nnz, void *scratch, void *stream) {
    RQ_TRY(check_batch(b));
    if (!rowptr || !scratch || !nnz) return fail(RQ_E_ARG, "rq_batch_conn_build: null argument");
    cudaStream_t st = as_stream(stream);
    int *err = scratch_err(scratch);
    if (!col) {
        RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        RQ_CUDA(cudaMemsetAsync(rowptr, 0, sizeof(int64_t), st));
        k_batch_conn_count<<<grid_rows(b->D, 6), kThreads, 0, st>>>(*b, rowptr + 1, err);
        RQ_CUDA(cudaGetLastError());
        RQ_TRY(scan_row_counts(rowptr + 1, b->D, scratch_scan(scratch), st));
        int h_err = 0;
        RQ_CUDA(cudaMemcpyAsync(nnz, rowptr + b->D, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        if (h_err) return fail(h_err, "rq_batch_conn_build: lookup failed");
        return RQ_OK;
    }
    if (!grp) return fail(RQ_E_ARG, "rq_batch_conn_build: grp is null");
    k_batch_conn_fill<<<grid_rows(b->D, 6), kThreads, 0, st>>>(*b, rowptr, col, grp, err);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_batch_matvec(const rq_batch_t *b, int32_t vtype, const void *x, void *y,
                           void *scratch, void *stream) {
    RQ_TRY(check_batch(b));
    if (!x || !y || x == y) return fail(RQ_E_ARG, "rq_batch_matvec: x and y must be distinct");
    if ((vtype == RQ_F32 || vtype == RQ_F64) && !b->terms.is_real)
        return fail(RQ_E_ARG, "rq_batch_matvec: real vectors need real coefficients");
    return batch_matvec_dispatch(*b, vtype, x, y, scratch, as_stream(stream), nullptr, 0, nullptr);
}
