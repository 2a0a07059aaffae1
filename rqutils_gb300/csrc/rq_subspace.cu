// Subspace construction and per-group lookups:
//   rq_subspace_build  -- strict-increase check, empty-key choice, hash table, sector filter
//   rq_xsource         -- get_xsource (rqutils/sqd.py:448-503) for any number of X masks
//   rq_diagonal        -- get_diagonal (rqutils/sqd.py:554-575), stopping at the first zero
#include <string>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {

namespace {

__global__ void k_check_sorted(const uint64_t *__restrict__ s, int64_t D, int *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i + 1 < D;
         i += (int64_t)gridDim.x * blockDim.x)
        if (s[i] >= s[i + 1]) atomicExch(flag, 1);
}

// First index i with s[i + 1] != s[i] + 1 (only needed when both 0 and the top key are states).
// One atomic per block after a block-wide minimum.
__global__ void k_first_gap(const uint64_t *__restrict__ s, int64_t D, unsigned long long *gap) {
    __shared__ unsigned long long best;
    if (threadIdx.x == 0) best = ~0ULL;
    __syncthreads();
    unsigned long long mine = ~0ULL;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i + 1 < D;
         i += (int64_t)gridDim.x * blockDim.x)
        if (s[i + 1] != s[i] + 1 && (unsigned long long)i < mine) mine = (unsigned long long)i;
    if (mine != ~0ULL) atomicMin(&best, mine);
    __syncthreads();
    if (threadIdx.x == 0 && best != ~0ULL) atomicMin(gap, best);
}

__global__ void k_fill_u64(uint64_t *p, int64_t n, uint64_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Insert every state into its bucket chain: claim the first empty slot with a CAS.  Keys are
// distinct, so a failed CAS always means "occupied by another key".  Slots of a bucket are
// claimed in order, which keeps the occupied slots a prefix of the bucket.
// presence bitmap: bit (hash(key) >> (32 - pbits)) for every key
template <int KB>
__global__ void k_pmap_build(const uint64_t *__restrict__ keys, int64_t D, uint32_t *pmap, int pbits) {
    __shared__ uint32_t T[kHashTableWords];
    init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t idx = lin_hash(T, keys[i], KeyWidth<KB>::kNbytes) >> (32 - pbits);
        atomicOr(pmap + (idx >> 5), 1u << (idx & 31));
    }
}

template <int KB>
__global__ void __launch_bounds__(kThreads)
k_hash_insert(const uint64_t *__restrict__ states, int64_t D, void *keys, int32_t *vals, int hbits,
              uint64_t empty, int *err) {
    __shared__ uint32_t T[kHashTableWords];
    init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    constexpr int kSlots = kBucketSlots;
    const uint32_t mask = (1u << hbits) - 1u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = states[i];
        uint32_t b = bucket_from_hash(lin_hash(T, key, KeyWidth<KB>::kNbytes), hbits);
        bool done = false;
        for (uint32_t n = 0; n <= mask && !done; ++n) {
            for (int s = 0; s < kSlots; ++s) {
                const size_t slot = (size_t)b * kSlots + s;
                bool won;
                if (KB == 64) {
                    unsigned long long *p = static_cast<unsigned long long *>(keys) + slot;
                    won = atomicCAS(p, (unsigned long long)empty, (unsigned long long)key) ==
                          (unsigned long long)empty;
                } else {
                    unsigned int *p = static_cast<unsigned int *>(keys) + slot;
                    won = atomicCAS(p, (unsigned int)empty, (unsigned int)key) == (unsigned int)empty;
                }
                if (won) {
                    vals[slot] = (int32_t)i;
                    done = true;
                    break;
                }
            }
            b = (b + 1) & mask;
        }
        if (!done) atomicExch(err, RQ_E_TABLE);
    }
}

// Highest differing bit of neighbouring sorted states: hist[h] counts the i with
// 63 - clz(s[i] ^ s[i - 1]) == h.  The number of distinct prefixes s >> b is then
// 1 + sum_{h >= b} hist[h] for every b at once.
__global__ void k_prefix_hist(const uint64_t *__restrict__ s, int64_t D,
                              unsigned long long *__restrict__ hist) {
    __shared__ unsigned int h[64];
    if (threadIdx.x < 64) h[threadIdx.x] = 0u;
    __syncthreads();
    for (int64_t i = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[63 - __clzll((long long)(s[i] ^ s[i - 1]))], 1u);
    __syncthreads();
    if (threadIdx.x < 64 && h[threadIdx.x]) atomicAdd(hist + threadIdx.x, (unsigned long long)h[threadIdx.x]);
}

// Line filter: for every state s with h = hash(s), word (h mod 2^lwbits) >> 5 of line
// hash(s >> lshift) >> (32 - lbits), bits h mod 32 and h >> 27 of that word (two bits of one word:
// a probe loads one word and a miss passes both tests with probability ~(1/64)^2).  Both hashes are
// the GF(2)-linear lookup hash, so a target's line, word and bits follow from the row's and the X
// mask's by XOR.
template <int KB>
__global__ void __launch_bounds__(kThreads)
k_line_build(const uint64_t *__restrict__ s, int64_t D, uint32_t *__restrict__ lmap, int lbits,
             int lwbits, int lshift) {
    __shared__ uint32_t T[kHashTableWords];
    init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    const uint32_t bmask = (1u << lwbits) - 1u;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = s[i];
        const uint32_t line = lin_hash(T, lshift < 64 ? k >> lshift : 0ULL, KeyWidth<KB>::kNbytes) >> (32 - lbits);
        const uint32_t h = lin_hash(T, k, KeyWidth<KB>::kNbytes);
        atomicOr(lmap + ((size_t)line << (lwbits - 5)) + ((h & bmask) >> 5), (1u << (h & 31)) | (1u << (h >> 27)));
    }
}

__global__ void k_fill_u32(uint32_t *p, int64_t n, uint32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void k_filter_build(const uint64_t *__restrict__ s, int64_t D, uint64_t fa, uint64_t fb,
                               uint32_t *bits) {
    __shared__ uint32_t loc[RQ_FILTER_WORDS];
    for (int w = threadIdx.x; w < RQ_FILTER_WORDS; w += blockDim.x) loc[w] = 0u;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = s[i];
        const int bit = __popcll(v & fa) * 65 + __popcll(v & fb);
        atomicOr(&loc[bit >> 5], 1u << (bit & 31));
    }
    __syncthreads();
    for (int w = threadIdx.x; w < RQ_FILTER_WORDS; w += blockDim.x)
        if (loc[w]) atomicOr(bits + w, loc[w]);
}

constexpr int kSample = 2048;  // shared-memory sample size of the binary-search lookup

template <int LK, int KB>
__global__ void __launch_bounds__(kThreads)
k_xsource(const rq_subspace_t S, const uint64_t *__restrict__ xm, int J, int32_t *__restrict__ out,
          int *err) {
    __shared__ uint32_t fb[RQ_FILTER_WORDS];
    __shared__ uint64_t samp[LK == RQ_LOOKUP_BSEARCH ? kSample : 1];
    __shared__ uint32_t T[LK == RQ_LOOKUP_HASH ? kHashTableWords : 1];
    for (int w = threadIdx.x; w < RQ_FILTER_WORDS; w += blockDim.x) fb[w] = S.fbits[w];
    const int ns = (int)(S.D < kSample ? S.D : kSample);
    if (LK == RQ_LOOKUP_BSEARCH)
        for (int k = threadIdx.x; k < ns; k += blockDim.x) samp[k] = S.states[((int64_t)k * S.D) / ns];
    if (LK == RQ_LOOKUP_HASH) init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    const int64_t total = (int64_t)J * S.D;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx / S.D);
        const int64_t i = idx - (int64_t)j * S.D;
        const uint64_t t = __ldg(S.states + i) ^ __ldg(xm + j);
        int m = -1;
        if (sector_ok(fb, S.fmask_a, S.fmask_b, t)) {
            if (LK == RQ_LOOKUP_HASH) {
                if (KB == 64 || (t >> 32) == 0)
                    m = lookup_hash_at<KB>(S, t, bucket_from_hash(lin_hash(T, t, KeyWidth<KB>::kNbytes),
                                                                  S.hbits), err);
            } else {
                m = lookup_bsearch(S, samp, ns, t);
            }
        }
        out[idx] = m;
    }
}

// get_diagonal with the reference's loop: terms in order, stop at the first zero coefficient.
__global__ void __launch_bounds__(kThreads)
k_diagonal(const uint64_t *__restrict__ s, int64_t D, const uint64_t *__restrict__ z,
           const double *__restrict__ c, int K, double2 *__restrict__ out) {
    constexpr int kChunk = 1024;
    __shared__ uint64_t zs[kChunk];
    __shared__ double cr[kChunk], ci[kChunk];
    __shared__ int kstop;
    if (threadIdx.x == 0) kstop = K;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x)
        if (c[2 * k] == 0. && c[2 * k + 1] == 0.) atomicMin(&kstop, k);
    __syncthreads();
    const int kend = kstop;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const uint64_t v = (i < D) ? s[i] : 0;
        double re = 0., im = 0.;
        for (int k0 = 0; k0 < kend; k0 += kChunk) {
            const int n = min(kChunk, kend - k0);
            __syncthreads();
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                zs[k] = z[k0 + k];
                cr[k] = c[2 * (k0 + k)];
                ci[k] = c[2 * (k0 + k) + 1];
            }
            __syncthreads();
            for (int k = 0; k < n; ++k) {
                const double sg = (__popcll(v & zs[k]) & 1) ? -1. : 1.;
                re += sg * cr[k];
                if (ci[k] != 0.) im += sg * ci[k];
            }
        }
        if (i < D) out[i] = make_double2(re, im);
    }
}

int grid_for(int64_t n, int per_sm = 8) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

// Strict-increase check, empty-key choice and hash insertion for a sorted key array; shared by
// rq_subspace_build and rq_batch_build.  `flag` and `gap` are device scratch words.
int build_key_table(const uint64_t *keys, int64_t D, int key_bits, bool hash, void *hkeys,
                    int32_t *hvals, int hbits, uint64_t *empty_out, int *flag,
                    unsigned long long *gap, cudaStream_t st, uint32_t *pmap, int pbits) {
    // buckets (keys) and their four row indices are read as vectors
    if (hash && (reinterpret_cast<uintptr_t>(hkeys) % 16 != 0 || reinterpret_cast<uintptr_t>(hvals) % 16 != 0))
        return fail(RQ_E_ARG, "hash table arrays (hkeys, hvals) must be 16-byte aligned");
    RQ_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    RQ_CUDA(cudaMemsetAsync(gap, 0xff, sizeof(unsigned long long), st));
    k_check_sorted<<<grid_for(D), kThreads, 0, st>>>(keys, D, flag);
    RQ_CUDA(cudaGetLastError());
    int h_flag = 0;
    unsigned long long h_gap = 0;
    uint64_t first = 0, last = 0;
    RQ_CUDA(cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaMemcpyAsync(&first, keys, 8, cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaMemcpyAsync(&last, keys + (D - 1), 8, cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    if (h_flag) return fail(RQ_E_UNSORTED, "keys are not strictly increasing");
    const uint64_t top = key_bits == 32 ? 0xFFFFFFFFULL : ~0ULL;
    if (key_bits == 32 && last > top)
        return fail(RQ_E_RANGE, "key_bits = 32 needs every state < 2^32");
    uint64_t empty;
    if (last != top) {
        empty = top;
    } else if (first != 0ULL) {
        empty = 0ULL;
    } else {  // both extremes present: the first gap exists because D < 2^64
        k_first_gap<<<grid_for(D), kThreads, 0, st>>>(keys, D, gap);
        RQ_CUDA(cudaMemcpyAsync(&h_gap, gap, sizeof(h_gap), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        uint64_t below = 0;
        RQ_CUDA(cudaMemcpy(&below, keys + h_gap, 8, cudaMemcpyDeviceToHost));
        empty = below + 1;
    }
    *empty_out = empty;
    RQ_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    if (hash) {
        const int64_t nslots = int64_t(kBucketSlots) << hbits;
        if (key_bits == 64) {
            k_fill_u64<<<grid_for(nslots), kThreads, 0, st>>>(static_cast<uint64_t *>(hkeys), nslots,
                                                              empty);
            k_hash_insert<64><<<grid_for(D), kThreads, 0, st>>>(keys, D, hkeys, hvals, hbits, empty,
                                                                flag);
        } else {
            k_fill_u32<<<grid_for(nslots), kThreads, 0, st>>>(static_cast<uint32_t *>(hkeys), nslots,
                                                              (uint32_t)empty);
            k_hash_insert<32><<<grid_for(D), kThreads, 0, st>>>(keys, D, hkeys, hvals, hbits, empty,
                                                                flag);
        }
        RQ_CUDA(cudaGetLastError());
        if (pmap && pbits > 0) {
            RQ_CUDA(cudaMemsetAsync(pmap, 0, ((size_t)1 << pbits) / 8, st));
            if (key_bits == 64)
                k_pmap_build<64><<<grid_for(D), kThreads, 0, st>>>(keys, D, pmap, pbits);
            else
                k_pmap_build<32><<<grid_for(D), kThreads, 0, st>>>(keys, D, pmap, pbits);
            RQ_CUDA(cudaGetLastError());
        }
        int h_err = 0;
        RQ_CUDA(cudaMemcpyAsync(&h_err, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        if (h_err) return fail(RQ_E_TABLE, "hash insertion failed");
    }
    return RQ_OK;
}

}  // namespace rq

using namespace rq;

RQ_API int rq_subspace_sizes(int64_t D, int32_t key_bits, int32_t *hbits) {
    if (!hbits || D < 1) return fail(RQ_E_ARG, "rq_subspace_sizes: D must be >= 1");
    if (key_bits != 32 && key_bits != 64) return fail(RQ_E_ARG, "rq_subspace_sizes: key_bits must be 32 or 64");
    int b = 1;
    while ((int64_t(1) << b) * kBucketSlots < 8 * D) ++b;  // load factor <= 1/8
    if (b > 31) return fail(RQ_E_RANGE, "rq_subspace_sizes: D too large");
    *hbits = b;
    return RQ_OK;
}

RQ_API int rq_line_filter_bits(int64_t D, int32_t lwbits, int32_t *lbits) {
    if (!lbits || D < 1 || lwbits < 8 || lwbits > 10)
        return fail(RQ_E_ARG, "rq_line_filter_bits: D >= 1 and 8 <= lwbits <= 10");
    const int64_t per = int64_t(1) << (lwbits - 7);  // states per line on average
    const int64_t lines = (D + per - 1) / per;
    int b = 1;
    while ((int64_t(1) << b) < lines) ++b;
    // at most 2^(37 - lwbits) lines, so that the index of a word (line << (lwbits - 5) | word in
    // the line) fits 32 bits; only subspaces of more than 2^29 states fill their lines fuller
    if (b > 37 - lwbits) b = 37 - lwbits;
    *lbits = b;
    return RQ_OK;
}

RQ_API int rq_presence_bits(int64_t D, int32_t key_bits, int32_t *pbits) {
    if (!pbits) return fail(RQ_E_ARG, "rq_presence_bits: null argument");
    int32_t hb = 0;
    RQ_TRY(rq_subspace_sizes(D, key_bits, &hb));
    const double table = (double)(key_bits / 8) * kBucketSlots * (double)(int64_t(1) << hb);
    *pbits = table <= 64.0 * (1 << 20) ? 0 : (hb + 2 < 29 ? hb + 2 : 29);
    if (*pbits != 0 && *pbits < hb) *pbits = hb;
    return RQ_OK;
}

RQ_API int rq_subspace_build(rq_subspace_t *sub, void *scratch, void *stream) {
    if (!sub || !sub->states || !scratch) return fail(RQ_E_ARG, "rq_subspace_build: null argument");
    const int64_t D = sub->D;
    if (D < 1 || D >= (int64_t(1) << 31))
        return fail(RQ_E_RANGE, "rq_subspace_build: D must be in [1, 2^31)");
    if (sub->lookup != RQ_LOOKUP_HASH && sub->lookup != RQ_LOOKUP_BSEARCH)
        return fail(RQ_E_ARG, "rq_subspace_build: lookup must be RQ_LOOKUP_HASH or RQ_LOOKUP_BSEARCH");
    if (!sub->fbits) return fail(RQ_E_ARG, "rq_subspace_build: fbits is null");
    if (sub->key_bits != 32 && sub->key_bits != 64)
        return fail(RQ_E_ARG, "rq_subspace_build: key_bits must be 32 or 64");
    const int slots = kBucketSlots;
    if (sub->lookup == RQ_LOOKUP_HASH) {
        if (!sub->hkeys || !sub->hvals || sub->hbits < 1 || sub->hbits > 31)
            return fail(RQ_E_ARG, "rq_subspace_build: hash buffers missing or hbits out of range");
        if ((int64_t(slots) << sub->hbits) < D + 1)
            return fail(RQ_E_ARG, "rq_subspace_build: hash table too small for D");
    }
    cudaStream_t st = as_stream(stream);
    int *flag = scratch_err(scratch);
    unsigned long long *gap = reinterpret_cast<unsigned long long *>(scratch);
    if (sub->lookup == RQ_LOOKUP_HASH && sub->lmap &&
        (sub->lbits < 1 || sub->lwbits < 8 || sub->lwbits > 10 || sub->lbits + sub->lwbits > 37))
        return fail(RQ_E_ARG, "rq_subspace_build: line filter needs 8 <= lwbits <= 10, 1 <= lbits <= 37 - lwbits");
    if (sub->lookup == RQ_LOOKUP_HASH && sub->pbits != 0 &&
        (!sub->pmap || sub->pbits < 5 || sub->pbits > 32 || sub->pbits < sub->hbits))
        return fail(RQ_E_ARG, "rq_subspace_build: presence bitmap missing or pbits out of range");
    const int rc = build_key_table(sub->states, D, sub->key_bits, sub->lookup == RQ_LOOKUP_HASH,
                                   sub->hkeys, sub->hvals, sub->hbits, &sub->empty_key, flag, gap,
                                   st, sub->pbits ? sub->pmap : nullptr, sub->pbits);
    if (rc != RQ_OK) return fail(rc, std::string("rq_subspace_build: ") + rq_last_error());
    if (sub->lookup == RQ_LOOKUP_HASH && sub->lmap) {
        // prefix shift: the largest b with about 2^(lwbits - 5) states per distinct s >> b
        // (the histogram sits in the reduction partials of the scratch, past the reduction
        // counter, which must stay zero)
        unsigned long long *hist = reinterpret_cast<unsigned long long *>(
            static_cast<char *>(scratch_reduce(scratch)) + 16);
        RQ_CUDA(cudaMemsetAsync(hist, 0, 64 * sizeof(unsigned long long), st));
        k_prefix_hist<<<grid_for(D), kThreads, 0, st>>>(sub->states, D, hist);
        RQ_CUDA(cudaGetLastError());
        unsigned long long h[64];
        RQ_CUDA(cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        const double per = (double)(1 << (sub->lwbits - 5));
        int b = 0;
        unsigned long long above = 0;  // distinct prefixes at shift b, minus one
        for (int k = 63; k >= 0; --k) above += h[k];
        for (int c = 1; c <= sub->key_bits; ++c) {
            above -= h[c - 1];
            if ((double)D > per * (double)(above + 1)) break;
            b = c;
        }
        sub->lshift = b;
        const size_t bytes = (size_t)1 << (sub->lbits + sub->lwbits - 3);
        RQ_CUDA(cudaMemsetAsync(sub->lmap, 0, bytes, st));
        if (sub->key_bits == 64)
            k_line_build<64><<<grid_for(D), kThreads, 0, st>>>(sub->states, D, sub->lmap,
                                                                sub->lbits, sub->lwbits, b);
        else
            k_line_build<32><<<grid_for(D), kThreads, 0, st>>>(sub->states, D, sub->lmap,
                                                                sub->lbits, sub->lwbits, b);
        RQ_CUDA(cudaGetLastError());
    }
    RQ_CUDA(cudaMemsetAsync(sub->fbits, 0, RQ_FILTER_WORDS * sizeof(uint32_t), st));
    k_filter_build<<<grid_for(D), kThreads, 0, st>>>(sub->states, D, sub->fmask_a, sub->fmask_b,
                                                      sub->fbits);
    RQ_CUDA(cudaGetLastError());
    // one sector (a single bit of the bitset): the matrix-free kernel then tests two popcounts
    uint32_t fb[RQ_FILTER_WORDS];
    RQ_CUDA(cudaMemcpyAsync(fb, sub->fbits, sizeof(fb), cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    int nbits = 0, bit = -1;
    for (int w = 0; w < RQ_FILTER_WORDS; ++w)
        for (int k = 0; k < 32; ++k)
            if ((fb[w] >> k) & 1u) {
                ++nbits;
                bit = w * 32 + k;
            }
    sub->fpoint = ((sub->fmask_a | sub->fmask_b) != 0 && nbits == 1) ? bit : -1;
    return RQ_OK;
}

RQ_API int rq_xsource(const rq_subspace_t *sub, const uint64_t *xmask, int32_t J, int32_t *out,
                      void *stream) {
    if (!sub || !xmask || !out || J < 0) return fail(RQ_E_ARG, "rq_xsource: bad arguments");
    if (J == 0) return RQ_OK;
    cudaStream_t st = as_stream(stream);
    const int64_t total = (int64_t)J * sub->D;
    const int g = grid_for(total);
    // the error flag of a hash chain that never ends is dropped here (the table was validated
    // at build time); a null pointer tells the lookup not to report
    if (sub->lookup == RQ_LOOKUP_HASH && sub->key_bits == 64)
        k_xsource<RQ_LOOKUP_HASH, 64><<<g, kThreads, 0, st>>>(*sub, xmask, J, out, nullptr);
    else if (sub->lookup == RQ_LOOKUP_HASH)
        k_xsource<RQ_LOOKUP_HASH, 32><<<g, kThreads, 0, st>>>(*sub, xmask, J, out, nullptr);
    else if (sub->lookup == RQ_LOOKUP_BSEARCH)
        k_xsource<RQ_LOOKUP_BSEARCH, 64><<<g, kThreads, 0, st>>>(*sub, xmask, J, out, nullptr);
    else
        return fail(RQ_E_ARG, "rq_xsource: unsupported lookup");
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_diagonal(const uint64_t *states, int64_t D, const uint64_t *zmask, const double *coef,
                       int32_t K, double *out, void *stream) {
    if (!states || !out || D < 1 || K < 0 || (K > 0 && (!zmask || !coef)))
        return fail(RQ_E_ARG, "rq_diagonal: bad arguments");
    cudaStream_t st = as_stream(stream);
    k_diagonal<<<grid_for(D, 4), kThreads, 0, st>>>(states, D, zmask, coef, K,
                                                   reinterpret_cast<double2 *>(out));
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}
