// Sample front end: pack 0/1 rows into uint64 states and sort + deduplicate them on the device
// (the reference's uniquify_states, sqd.py:414-445, a lexsort of packed rows plus unique).
//
// Sort: least-significant-digit radix sort with 8-bit digits, skipping every digit on which all
// keys agree (a 32-qubit sample needs at most 4 passes).  A pass is a histogram kernel (one
// 4096-key tile per block, shared-memory counters, written digit-major), an exclusive scan of the
// 256 x tiles counters, and a stable scatter: each warp ranks its keys with __match_any_sync, the
// warps of a block add their counts for the same digit in order, and a per-digit running base
// carries the order across the tile's 16 rounds.  Unique: flags, inclusive scan, compaction.
#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {

int scan_row_counts(int64_t *v, int64_t D, int64_t *bsum, cudaStream_t st);

namespace {

constexpr int kSortThreads = 256;
constexpr int kRounds = 16;
constexpr int64_t kTile = (int64_t)kSortThreads * kRounds;  // 4096 keys per block

int64_t tiles_of(int64_t n) { return (n + kTile - 1) / kTile; }

__global__ void k_pack(const uint8_t *__restrict__ bits, int64_t rows, int n, int64_t stride,
                       uint64_t *__restrict__ out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t *row = bits + r * stride;
        uint64_t s = 0;
        for (int c = 0; c < n; ++c)  // column 0 is qubit n - 1
            if (row[c]) s |= 1ULL << (n - 1 - c);
        out[r] = s;
    }
}

// bits on which the keys differ: OR ^ AND over all keys
__global__ void k_or_and(const uint64_t *__restrict__ k, int64_t n, unsigned long long *oa) {
    unsigned long long o = 0ULL, a = ~0ULL;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        o |= k[i];
        a &= k[i];
    }
    for (int s = 16; s > 0; s >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, s);
        a &= __shfl_xor_sync(0xffffffffu, a, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicOr(oa, o);
        atomicAnd(oa + 1, a);
    }
}

// counts[1 + d * tiles + b] = keys of tile b with digit d
__global__ void __launch_bounds__(kSortThreads) k_hist(const uint64_t *__restrict__ src, int64_t n, int shift,
                                                       int64_t tiles, int64_t *__restrict__ counts) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int r = 0; r < kRounds; ++r) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(int)((src[i] >> shift) & 255ULL)], 1);
    }
    __syncthreads();
    counts[1 + (int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// stable scatter by digit; base[d * tiles + b] = first output position of (digit d, tile b)
__global__ void __launch_bounds__(kSortThreads) k_scatter(const uint64_t *__restrict__ src, uint64_t *__restrict__ dst,
                                                          int64_t n, int shift, int64_t tiles,
                                                          const int64_t *__restrict__ base) {
    __shared__ unsigned long long run[256];
    __shared__ int wcnt[kSortThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    run[tid] = (unsigned long long)base[(int64_t)tid * tiles + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int r = 0; r < kRounds; ++r) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + tid;
        const bool valid = i < n;
        const uint64_t k = valid ? src[i] : 0ULL;
        const int d = valid ? (int)((k >> shift) & 255ULL) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        const bool leader = (__ffs(peers) - 1) == lane;
        if (valid && leader) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned long long pos = run[d] + (unsigned long long)rank;
            for (int w = 0; w < warp; ++w) pos += (unsigned long long)wcnt[w][d];
            dst[pos] = k;
        }
        __syncthreads();
        if (valid && leader) {
            atomicAdd(&run[d], (unsigned long long)__popc(peers));
            wcnt[warp][d] = 0;
        }
        __syncthreads();
    }
}

// The same two passes for a permutation: element i stands for index perm[i], its digit is taken
// from key[perm[i]], and the scatter moves the index (a stable sort of the indices by the key).
__global__ void __launch_bounds__(kSortThreads) k_hist_perm(const uint64_t *__restrict__ key,
                                                            const int64_t *__restrict__ perm, int64_t n,
                                                            int shift, int64_t tiles,
                                                            int64_t *__restrict__ counts) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int r = 0; r < kRounds; ++r) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(int)((key[perm[i]] >> shift) & 255ULL)], 1);
    }
    __syncthreads();
    counts[1 + (int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) k_scatter_perm(const uint64_t *__restrict__ key,
                                                               const int64_t *__restrict__ src,
                                                               int64_t *__restrict__ dst, int64_t n,
                                                               int shift, int64_t tiles,
                                                               const int64_t *__restrict__ base) {
    __shared__ unsigned long long run[256];
    __shared__ int wcnt[kSortThreads / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    run[tid] = (unsigned long long)base[(int64_t)tid * tiles + blockIdx.x];
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    const int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int r = 0; r < kRounds; ++r) {
        const int64_t i = t0 + (int64_t)r * kSortThreads + tid;
        const bool valid = i < n;
        const int64_t e = valid ? src[i] : 0;
        const int d = valid ? (int)((key[e] >> shift) & 255ULL) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        const bool leader = (__ffs(peers) - 1) == lane;
        if (valid && leader) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned long long pos = run[d] + (unsigned long long)rank;
            for (int w = 0; w < warp; ++w) pos += (unsigned long long)wcnt[w][d];
            dst[pos] = e;
        }
        __syncthreads();
        if (valid && leader) {
            atomicAdd(&run[d], (unsigned long long)__popc(peers));
            wcnt[warp][d] = 0;
        }
        __syncthreads();
    }
}

__global__ void k_iota64(int64_t *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = i;
}

__global__ void k_or_and_perm(const uint64_t *__restrict__ k, int64_t n, unsigned long long *oa) {
    unsigned long long o = 0ULL, a = ~0ULL;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        o |= k[i];
        a &= k[i];
    }
    for (int s = 16; s > 0; s >>= 1) {
        o |= __shfl_xor_sync(0xffffffffu, o, s);
        a &= __shfl_xor_sync(0xffffffffu, a, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicOr(oa, o);
        atomicAnd(oa + 1, a);
    }
}

__global__ void k_flags(const uint64_t *__restrict__ s, int64_t n, int64_t *__restrict__ fl) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        fl[i] = (i == 0 || s[i] != s[i - 1]) ? 1 : 0;
}

__global__ void k_compact(const uint64_t *__restrict__ s, int64_t n, const int64_t *__restrict__ incl,
                          uint64_t *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (i == 0 || s[i] != s[i - 1]) out[incl[i] - 1] = s[i];
}

struct SortLayout {
    int64_t tiles;
    size_t oa, alt, counts, flags, bsum, total;
};

SortLayout sort_layout(int64_t n) {
    SortLayout L{};
    L.tiles = tiles_of(n);
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off += (b + 255) & ~size_t(255);
        return o;
    };
    const int64_t ncnt = 256 * L.tiles + 1;
    const int64_t nscan = ncnt > n ? ncnt : n;
    L.oa = take(16);
    L.alt = take((size_t)n * 8);
    L.counts = take((size_t)ncnt * 8);
    L.flags = take((size_t)n * 8);
    L.bsum = take((size_t)((nscan + 1023) / 1024 + 1) * 8);
    L.total = off;
    return L;
}

int grid_for(int64_t n) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

// Stable sort of the indices 0..n-1 by a key of nw 64-bit words (words[0] the least significant),
// left in perm; least-significant-digit passes over the 8-bit digits on which the keys differ.
// Scratch: alt [n], counts [256 * tiles + 1], bsum (scan block sums), oa [2] words.
size_t sort_perm_scratch(int64_t n) {
    const int64_t tiles = tiles_of(n);
    const int64_t ncnt = 256 * tiles + 1;
    return ((size_t)n * 8 + 255) / 256 * 256 + ((size_t)ncnt * 8 + 255) / 256 * 256 +
           ((size_t)((ncnt + 1023) / 1024 + 1) * 8 + 255) / 256 * 256 + 256;
}

int sort_perm(const uint64_t *const *words, int nw, int64_t n, int64_t *perm, void *scratch,
              cudaStream_t st) {
    if (n < 1) return RQ_OK;
    const int64_t tiles = tiles_of(n);
    const int64_t ncnt = 256 * tiles + 1;
    char *w = static_cast<char *>(scratch);
    int64_t *alt = reinterpret_cast<int64_t *>(w);
    w += ((size_t)n * 8 + 255) / 256 * 256;
    int64_t *counts = reinterpret_cast<int64_t *>(w);
    w += ((size_t)ncnt * 8 + 255) / 256 * 256;
    int64_t *bsum = reinterpret_cast<int64_t *>(w);
    w += ((size_t)((ncnt + 1023) / 1024 + 1) * 8 + 255) / 256 * 256;
    unsigned long long *oa = reinterpret_cast<unsigned long long *>(w);
    k_iota64<<<grid_for(n), kThreads, 0, st>>>(perm, n);
    RQ_CUDA(cudaGetLastError());
    int64_t *bufs[2] = {perm, alt};
    int cur = 0;
    for (int k = 0; k < nw; ++k) {
        const unsigned long long init[2] = {0ULL, ~0ULL};
        RQ_CUDA(cudaMemcpyAsync(oa, init, sizeof(init), cudaMemcpyHostToDevice, st));
        k_or_and_perm<<<grid_for(n), kThreads, 0, st>>>(words[k], n, oa);
        unsigned long long h_oa[2];
        RQ_CUDA(cudaMemcpyAsync(h_oa, oa, sizeof(h_oa), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        const uint64_t vary = h_oa[0] ^ h_oa[1];
        for (int p = 0; p < 8; ++p) {
            if (!((vary >> (8 * p)) & 0xFFULL)) continue;
            RQ_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t), st));
            k_hist_perm<<<(unsigned)tiles, kSortThreads, 0, st>>>(words[k], bufs[cur], n, 8 * p,
                                                                  tiles, counts);
            RQ_CUDA(cudaGetLastError());
            RQ_TRY(scan_row_counts(counts + 1, 256 * tiles, bsum, st));
            k_scatter_perm<<<(unsigned)tiles, kSortThreads, 0, st>>>(words[k], bufs[cur],
                                                                     bufs[cur ^ 1], n, 8 * p,
                                                                     tiles, counts);
            RQ_CUDA(cudaGetLastError());
            cur ^= 1;
        }
    }
    if (cur) RQ_CUDA(cudaMemcpyAsync(perm, alt, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
    return RQ_OK;
}

}  // namespace rq

using namespace rq;

RQ_API int rq_pack_states(const uint8_t *bits, int64_t rows, int32_t n, int64_t row_stride, uint64_t *out,
                          void *stream) {
    if (!bits || !out || rows < 1 || n < 1 || n > 64 || row_stride < n)
        return fail(RQ_E_ARG, "rq_pack_states: bad arguments");
    k_pack<<<grid_for(rows), kThreads, 0, as_stream(stream)>>>(bits, rows, n, row_stride, out);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_uniquify_scratch_size(int64_t n, size_t *bytes) {
    if (n < 1 || !bytes) return fail(RQ_E_ARG, "rq_uniquify_scratch_size: bad arguments");
    *bytes = sort_layout(n).total;
    return RQ_OK;
}

RQ_API int rq_uniquify(const uint64_t *in, int64_t n, uint64_t *out, int64_t *count, void *scratch,
                       void *stream) {
    if (!in || !out || !count || !scratch || n < 1 || in == out)
        return fail(RQ_E_ARG, "rq_uniquify: bad arguments");
    if (n >= (int64_t(1) << 40)) return fail(RQ_E_RANGE, "rq_uniquify: too many samples");
    const SortLayout L = sort_layout(n);
    char *w = static_cast<char *>(scratch);
    cudaStream_t st = as_stream(stream);
    unsigned long long *oa = reinterpret_cast<unsigned long long *>(w + L.oa);
    uint64_t *alt = reinterpret_cast<uint64_t *>(w + L.alt);
    int64_t *counts = reinterpret_cast<int64_t *>(w + L.counts);
    int64_t *fl = reinterpret_cast<int64_t *>(w + L.flags);
    int64_t *bsum = reinterpret_cast<int64_t *>(w + L.bsum);
    const unsigned long long init[2] = {0ULL, ~0ULL};
    RQ_CUDA(cudaMemcpyAsync(oa, init, sizeof(init), cudaMemcpyHostToDevice, st));
    k_or_and<<<grid_for(n), kThreads, 0, st>>>(in, n, oa);
    unsigned long long h_oa[2];
    RQ_CUDA(cudaMemcpyAsync(h_oa, oa, sizeof(h_oa), cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    const uint64_t vary = h_oa[0] ^ h_oa[1];
    int shifts[8], npass = 0;
    for (int p = 0; p < 8; ++p)
        if ((vary >> (8 * p)) & 0xFFULL) shifts[npass++] = 8 * p;
    // ping-pong so that the last pass writes alt; the compaction then writes out
    const uint64_t *src = in;
    uint64_t *bufs[2] = {(npass & 1) ? alt : out, (npass & 1) ? out : alt};
    const int64_t ncnt = 256 * L.tiles;
    for (int p = 0; p < npass; ++p) {
        uint64_t *dst = bufs[p & 1];
        RQ_CUDA(cudaMemsetAsync(counts, 0, sizeof(int64_t), st));
        k_hist<<<(unsigned)L.tiles, kSortThreads, 0, st>>>(src, n, shifts[p], L.tiles, counts);
        RQ_CUDA(cudaGetLastError());
        RQ_TRY(scan_row_counts(counts + 1, ncnt, bsum, st));
        k_scatter<<<(unsigned)L.tiles, kSortThreads, 0, st>>>(src, dst, n, shifts[p], L.tiles, counts);
        RQ_CUDA(cudaGetLastError());
        src = dst;
    }
    // src holds the sorted keys (alt after >= 1 pass, in when every key is equal)
    k_flags<<<grid_for(n), kThreads, 0, st>>>(src, n, fl);
    RQ_TRY(scan_row_counts(fl, n, bsum, st));
    k_compact<<<grid_for(n), kThreads, 0, st>>>(src, n, fl, out);
    RQ_CUDA(cudaGetLastError());
    RQ_CUDA(cudaMemcpyAsync(count, fl + n - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    return RQ_OK;
}
