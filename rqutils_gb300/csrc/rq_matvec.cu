// Pauli-sum matvec restricted to a sorted subspace (rqutils/sqd.py:578-684) and the full-space
// form (rqutils/paulis/symplectic.py:131-150).
//
// Row-side formula: (H x)[i] = sum_j d_j(S[i]) x[m_j(i)],  d_j(s) = sum_k c_jk (-1)^popcount(s & z_jk),
// S[m_j(i)] = S[i] ^ x_j (term dropped when absent).  One thread owns one row; the X masks,
// offsets, Z masks and coefficients of a tile of groups sit in shared memory and every thread of
// the block walks the same group sequence (broadcast reads).  Lookups of four groups are issued
// together (four independent 32-byte bucket loads in flight per thread).  d_j is only evaluated
// on a hit; the x = 0 group's diagonal is either read from a cached FP64 array or computed.
//
// Modes: FREE (lookups every call, cache_level (0, *)), CONN (cached (row -> source, group)
// lists, diagonals recomputed, cache_level (1, 0)), CSR (cached element values, (*, 2)).
#include <cmath>

#include "rq_common.cuh"
#include "rq_rows.cuh"
#include "rq_host.h"

namespace rq {

namespace {

constexpr int kGT = 512;      // max groups per shared-memory tile
constexpr int kKT = 2048;     // max terms per shared-memory tile
constexpr int kSample = 2048; // shared-memory sample of the binary-search lookup
constexpr int kFilterBytes = 544;

template <typename R>
struct Tile {
    uint64_t *xm;
    uint32_t *hx;  // linear hash of each X mask (hash-lookup kernel only)
    uint2 *gs;     // (low 32 bits of the X mask, its hash): one 8-byte read per group
    int32_t *off;
    uint64_t *zm;
    cx<R> *cf;
};

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

template <typename R>
__host__ __device__ inline size_t tile_bytes(int gt, int kt) {
    return align16((size_t)gt * 8) + align16((size_t)gt * 4) + align16((size_t)gt * 8) +
           align16((size_t)(gt + 1) * 4) + align16((size_t)kt * 8) + (size_t)kt * sizeof(cx<R>);
}

template <typename R>
__device__ inline Tile<R> carve(unsigned char *p, int gt, int kt) {
    Tile<R> t;
    t.xm = reinterpret_cast<uint64_t *>(p);
    p += align16((size_t)gt * 8);
    t.hx = reinterpret_cast<uint32_t *>(p);
    p += align16((size_t)gt * 4);
    t.gs = reinterpret_cast<uint2 *>(p);
    p += align16((size_t)gt * 8);
    t.off = reinterpret_cast<int32_t *>(p);
    p += align16((size_t)(gt + 1) * 4);
    t.zm = reinterpret_cast<uint64_t *>(p);
    p += align16((size_t)kt * 8);
    t.cf = reinterpret_cast<cx<R> *>(p);
    return t;
}

// Stage groups [g0, g1) into shared memory, g1 as large as the tile allows.  Returns g1, or -1
// when group g0 alone exceeds the tile.  Every thread of the block must call it.  With a hash
// table T the linear hash of each X mask is stored too.
template <typename R>
__device__ int load_tile(const rq_terms_t &T, int g0, int gt, int kt, const Tile<R> &tl,
                         int *s_g1, const uint32_t *htab = nullptr, int nbytes = 8) {
    __syncthreads();  // previous tile no longer in use; tables written before are visible
    if (threadIdx.x == 0) *s_g1 = g0;
    __syncthreads();
    const int base = T.toff[g0];
    const int gmax = min(T.J, g0 + gt);
    for (int g = g0 + 1 + threadIdx.x; g <= gmax; g += blockDim.x)
        if (T.toff[g] - base <= kt) atomicMax(s_g1, g);
    __syncthreads();
    const int g1 = *s_g1;
    if (g1 == g0) return -1;
    const int ng = g1 - g0;
    const int nk = T.toff[g1] - base;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        const uint64_t xv = T.xmask[g0 + g];
        tl.xm[g] = xv;
        if (htab) {
            const uint32_t h = lin_hash(htab, xv, nbytes);
            tl.hx[g] = h;
            tl.gs[g] = make_uint2((uint32_t)xv, h);
        }
    }
    for (int g = threadIdx.x; g <= ng; g += blockDim.x) tl.off[g] = T.toff[g0 + g] - base;
    for (int k = threadIdx.x; k < nk; k += blockDim.x) {
        tl.zm[k] = T.zmask[base + k];
        tl.cf[k] = {(R)T.coef[2 * (base + k)], (R)T.coef[2 * (base + k) + 1]};
    }
    __syncthreads();
    return g1;
}

// d_j(s) * xv accumulated into acc; the group's terms end at the first zero coefficient when
// stop_at_zero (subspace form) and run to the end otherwise (full-space form).
template <typename R>
__device__ __forceinline__ void add_group(const cx<R> *cf, const uint64_t *zm, int k0, int k1,
                                          uint64_t s, cx<R> xv, bool stop_at_zero, CAcc<R> &acc) {
    CAcc<R> d;
    for (int k = k0; k < k1; ++k) {
        const cx<R> c = cf[k];
        if (stop_at_zero && c.re == (R)0 && c.im == (R)0) break;
        if (__popcll(s & zm[k]) & 1) d.add({-c.re, -c.im});
        else d.add(c);
    }
    acc.add(cmul(d.get(), xv));
}

// Visit the hits of row state s over groups [g0, g1) (xm indexed by g - g0), skipping `skip`,
// calling on_hit(g, m) in ascending g.  Hash lookups hash each target in full (T: tables).
template <int LK, int KB, typename F>
__device__ __forceinline__ void for_hits(const rq_subspace_t &S, const uint32_t *fb,
                                         const uint64_t *samp, int ns, const uint32_t *T,
                                         const uint64_t *xm, int g0, int g1, int skip, uint64_t s,
                                         int *err, F &&on_hit) {
    for (int g = g0; g < g1; ++g) {
        if (g == skip) continue;
        const uint64_t t = s ^ xm[g - g0];
        int64_t m;
        if (LK == RQ_LOOKUP_IDENTITY) {
            m = (t < (uint64_t)S.D) ? (int64_t)t : -1;
        } else {
            if (!sector_ok(fb, S.fmask_a, S.fmask_b, t)) continue;
            if (LK == RQ_LOOKUP_HASH) {
                if (KB == 32 && (t >> 32) != 0) continue;
                const uint32_t h = lin_hash(T, t, KeyWidth<KB>::kNbytes);
                if (S.pbits > 0 && S.pmap && !present(S.pmap, h, S.pbits)) continue;
                m = lookup_hash_at<KB>(S, t, bucket_from_hash(h, S.hbits), err);
            } else {
                m = lookup_bsearch(S, samp, ns, t);
            }
        }
        if (m >= 0) on_hit(g, m);
    }
}

template <int LK>
__device__ inline void load_lookup_smem(const rq_subspace_t &S, uint32_t *fb, uint64_t *samp,
                                        int ns) {
    if (LK != RQ_LOOKUP_IDENTITY)
        for (int w = threadIdx.x; w < RQ_FILTER_WORDS; w += blockDim.x) fb[w] = S.fbits[w];
    if (LK == RQ_LOOKUP_BSEARCH)
        for (int k = threadIdx.x; k < ns; k += blockDim.x)
            samp[k] = S.states[((int64_t)k * S.D) / ns];
}

// ------------------------------------------------------------------------------------------
// FREE mode with the hash table: the hot kernel
// ------------------------------------------------------------------------------------------
// One thread per row.  Per row: h(s) once; per X group: t = s ^ x_j, sector filter,
// bucket = (h(s) ^ h(x_j)) >> shift, one bucket load.  The per-group data (x_j, h(x_j)) is read
// with broadcast shared-memory loads (every thread walks the same group sequence); the terms of
// a group are read from global memory only on a hit.  U bucket loads are issued together; the
// loop only marks "hot" groups (a key match, a full bucket, or a target equal to the empty key)
// in a 64-bit mask, resolved once per 64 groups so that the rare divergent work is not
// interleaved with the probes.  Each bucket load is one 16- or 32-byte read at a random address,
// one L1 wavefront per lane; at D = 2^20 (tables in L2) those wavefronts are the limit.
//
// With the line filter (rq_subspace_t.lmap) the probe is a bit test in a line chosen by the
// target's prefix t >> lshift: the rows of a warp are consecutive sorted states that share their
// high bits, so for one X group their targets share them too and the warp's probes fall in a few
// lines (one wavefront each) instead of one line per lane.  Set bits are resolved in the table.

// Group keys live in shared memory for the whole launch: (x_j, h(x_j)) packed as uint2 for 32-bit
// keys or as uint64 + uint32 arrays for 64-bit keys, then the line hash hl_j = h(x_j >> lshift)
// (12 or 16 B per group).  The x = 0 group is left out of the list (its diagonal is applied before
// the probes), so that the probe loop has no per-group skip test; resident index c is group
// c + (c >= diag_group).  Large J runs one 1024-thread block per SM so that up to
// max_resident_groups fit; above that the keys are streamed through in tiles.
template <int KB>
__host__ __device__ constexpr int max_resident_groups() {
    return KB == 32 ? 16384 : 12288;  // 192 KB of shared memory either way
}

template <int KB>
__host__ __device__ inline size_t group_key_bytes(int J) {
    return align16((size_t)J * 8) + (KB == 32 ? 0 : align16((size_t)J * 4)) + (size_t)J * 4;
}

template <int KB>
__host__ __device__ inline size_t group_line_offset(int kt) {
    return align16((size_t)kt * 8) + (KB == 32 ? 0 : align16((size_t)kt * 4));
}

// Sector filter of the hash kernel: none, the general (popcount a, popcount b) bitset, or the
// common case of a subspace in one sector (a single bit set: two popcount compares, no table).
enum { kFiltNone = 0, kFiltSet = 1, kFiltPoint = 2 };
// line filters of at most 2^25 bytes (32 MB, a quarter of GB300's L2) skip the sector test:
// measured faster without it at 16 MB (Hubbard D = 2^20: 0.089 against 0.107 ms) and slower at
// 64 MB (chemistry, 2^22 rows: 80.2 against 65.6 ms)
constexpr int kLineFilterL2Log2Bytes = 25;

// shared memory of the hash kernel: the sector bitset, the hash byte tables (64-bit keys use
// all eight) and, in dynamic shared memory, the resident group keys
__shared__ uint32_t hk_fb[RQ_FILTER_WORDS];
__shared__ uint32_t hk_htab[kHashTableWords];
extern __shared__ __align__(16) unsigned char hk_dyn[];

// Line-filter word of a key (a state or an X mask): the word index line << (lwbits - 5) | word
// within the line, line = h(k >> lshift) >> (32 - lbits), word = (h(k) mod 2^lwbits) >> 5.  Every
// step is linear over XOR, so the word of a target s ^ x is word(s) ^ word(x) (lbits + lwbits - 5
// <= 32 bits, rq_line_filter_bits).
__device__ __forceinline__ uint32_t line_word(uint32_t h, uint32_t hpre, const rq_subspace_t &S) {
    return ((hpre >> (32 - S.lbits)) << (S.lwbits - 5)) | ((h & ((1u << S.lwbits) - 1u)) >> 5);
}

// Group keys of resident indices [c0, c0 + cn) into shared-memory slots [0, cn); the layout holds
// kt slots (32-bit keys: (x, h(x)) pairs; 64-bit keys: x masks, then hashes; then, with the line
// filter, the line-filter words of the X masks).  Resident index c is group c + (c >= diag_group).
// All threads of the block call it.
template <int KB>
__device__ __forceinline__ void load_group_keys(const rq_terms_t &T, int c0, int cn, int kt,
                                                const rq_subspace_t &S) {
    constexpr int NB = KeyWidth<KB>::kNbytes;
    const int skip = T.diag_group;
    uint32_t *hl = reinterpret_cast<uint32_t *>(hk_dyn + group_line_offset<KB>(kt));
    for (int c = threadIdx.x; c < cn; c += blockDim.x) {
        const int j = c0 + c + (skip >= 0 && c0 + c >= skip);
        const uint64_t xv = T.xmask[j];
        const uint32_t h = T.xhash ? T.xhash[j] : lin_hash(hk_htab, xv, NB);
        if (KB == 32) {
            reinterpret_cast<uint2 *>(hk_dyn)[c] = make_uint2((uint32_t)xv, h);
        } else {
            reinterpret_cast<uint64_t *>(hk_dyn)[c] = xv;
            reinterpret_cast<uint32_t *>(hk_dyn + align16((size_t)kt * 8))[c] = h;
        }
        hl[c] = S.lmap ? line_word(h, lin_hash(hk_htab, S.lshift < 64 ? xv >> S.lshift : 0ULL, NB), S) : 0u;
    }
}

// Probes in flight per thread: four with key buckets (a 16- or 32-byte bucket per probe fills the
// 40 registers of six resident 256-thread blocks).  With the line filter (one 4-byte word per
// probe): 32 for 32-bit keys without a sector test, 16 in the 1024-thread kernel of 64-bit keys,
// 8 otherwise, 4 with the bitset sector test: the most that compile without new spills (ptxas -v).
// More probes in flight measured 5 % faster on the 64-qubit chemistry subspace (61.7 against
// 65.4 ms at 2^22 rows, one-bit filter) and the same on Hubbard.  A divisor of the 64 groups of a
// super-chunk.
constexpr int kKeyProbes = 4;

template <typename V, int KB, int FM, bool TL>
__host__ __device__ constexpr int line_probes() {
    return FM == kFiltSet ? 4 : (KB == 32 && FM == kFiltNone) ? 32 : (KB == 64 && TL) ? 16 : 8;
}

// LF: probe the line filter.  TL: the group keys may need streaming in tiles (1024-thread kernels
// only; with 256-thread blocks they always fit and the tile loop is one pass known at compile
// time).
template <typename V, int KB, int FM, bool LF, bool TL>
__device__ __forceinline__ void hash_rows(const rq_operator_t &op, const V *__restrict__ x,
                                          V *__restrict__ y, int *err, int pa0, int pb0) {
    using R = typename VT<V>::R;
    using K = typename KeyWidth<KB>::K;
    constexpr int NB = KeyWidth<KB>::kNbytes;
    constexpr int kBucketBytes = KeyWidth<KB>::kBucketBytes;
    constexpr int U = LF ? line_probes<V, KB, FM, TL>() : kKeyProbes;
    const rq_subspace_t &S = op.sub;
    const rq_terms_t &T = op.terms;
    const int64_t D = S.D;
    const int skip = T.diag_group;  // the x = 0 group is applied outside the probe loop
    const int nres = T.J - (skip >= 0 ? 1 : 0);  // groups of the probe loop
    // shared-memory slots: every group's keys when they fit (loaded once by the kernel), else
    // tiles of max_resident_groups streamed through for every row batch
    constexpr int kMaxRes = max_resident_groups<KB>();
    const int kt = (!TL || nres <= kMaxRes) ? nres : kMaxRes;
    const bool tiled = TL && nres > kt;
    const uint2 *gk32 = reinterpret_cast<const uint2 *>(hk_dyn);
    const uint64_t *gx64 = reinterpret_cast<const uint64_t *>(hk_dyn);
    const uint32_t *gh64 = reinterpret_cast<const uint32_t *>(hk_dyn + align16((size_t)kt * 8));
    const uint32_t *ghl = reinterpret_cast<const uint32_t *>(hk_dyn + group_line_offset<KB>(kt));
    const bool d0 = (op.diag0 != nullptr) && (skip >= 0);
    const K fa = (K)S.fmask_a, fbm = (K)S.fmask_b, empty = (K)S.empty_key;
    const int shift = 32 - S.hbits;
    // the line filter replaces the presence bitmap
    const uint32_t *pmap = (!LF && S.pbits > 0) ? S.pmap : nullptr;
    const int pshift = 32 - S.pbits;
    const unsigned char *keys = static_cast<const unsigned char *>(S.hkeys);
    const uint32_t *lmap = S.lmap;
    auto sector = [&](K t) -> bool {
        if (FM == kFiltPoint) {
            int pa, pb;
            if (sizeof(K) == 8) {
                pa = __popcll((unsigned long long)(t & fa));
                pb = __popcll((unsigned long long)(t & fbm));
            } else {
                pa = __popc((unsigned)(t & fa));
                pb = __popc((unsigned)(t & fbm));
            }
            return (pa == pa0) & (pb == pb0);
        }
        if (FM == kFiltSet) return sector_ok_k<K>(hk_fb, fa, fbm, t);
        return true;
    };
    // Every lane runs the same row batches and super-chunks, so that the warp can be
    // re-converged after each super-chunk's hot-group resolution; without the explicit
    // __syncwarp the lanes that took the rare path stay split from the rest for the remainder of
    // the row.  Lanes past D probe the last row again and store nothing.
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const bool active = i < D;
        const int64_t ir = active ? i : D - 1;
        const uint64_t s64 = __ldg(S.states + ir);
        const K s = (K)s64;
        const uint32_t hs = lin_hash(hk_htab, s64, NB);
        // the row's line-filter word: a target's word is wrow ^ hl[j], its bit (hs ^ h(x)) mod 32
        const uint32_t wrow = LF ? line_word(hs, lin_hash(hk_htab, S.lshift < 64 ? s64 >> S.lshift : 0ULL, NB), S) : 0u;
        CAcc<R> acc;
        const cx<R> xi = VT<V>::ld(x, ir);
        if (d0) {
            const R dv = (R)op.diag0[ir];
            acc.add({dv * xi.re, dv * xi.im});
        } else if (skip >= 0) {
            acc.add(cmul(group_diag<R>(T, skip, s64), xi));
        }
        for (int t0 = 0; TL ? t0 < nres : t0 < 1; t0 += TL ? kt : 1) {
            const int tn = TL ? min(kt, nres - t0) : nres;
            if (tiled) {
                __syncthreads();  // the previous tile is no longer read
                load_group_keys<KB>(T, t0, tn, kt, S);
                __syncthreads();
            }
            for (int gs0 = 0; gs0 < tn; gs0 += 64) {
                const int gs1 = min(tn, gs0 + 64);
                uint64_t hot = 0ULL;
                int g = gs0;
                for (; g + U <= gs1; g += U) {
                    K t[U];
                    uint32_t b[U], ln[U];
                    bool q[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        uint32_t hxg;
                        if (KB == 32) {
                            const uint2 e = gk32[g + u];
                            t[u] = s ^ (K)e.x;
                            hxg = e.y;
                        } else {
                            t[u] = s ^ (K)gx64[g + u];
                            hxg = gh64[g + u];
                        }
                        q[u] = sector(t[u]);
                        b[u] = hs ^ hxg;
                        if (LF) ln[u] = wrow ^ ghl[g + u];
                    }
                    if (pmap) {  // presence bitmap (L2-resident) in front of a table that is not
                        uint32_t pw[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const uint32_t idx = b[u] >> pshift;
                            pw[u] = q[u] ? __ldg(pmap + (idx >> 5)) : 0u;
                        }
#pragma unroll
                        for (int u = 0; u < U; ++u) q[u] = q[u] && ((pw[u] >> ((b[u] >> pshift) & 31)) & 1u);
                    }
                    uint32_t hb = 0u;  // hot bits of this batch, constant shifts
                    if (LF) {
                        // line filter: a hot lane's bit is set (a state, or another state's bit;
                        // the resolution below compares the keys).  A lane whose target fails
                        // the sector filter reads no word: the zero word it keeps is never hot,
                        // so q need not stay live across the loads.
                        uint32_t w[U];
#pragma unroll
                        for (int u = 0; u < U; ++u)
                            w[u] = load_word(lmap + ln[u], q[u]);
#pragma unroll
                        for (int u = 0; u < U; ++u)
                            if ((w[u] >> (b[u] & 31u)) & (w[u] >> (b[u] >> 27)) & 1u) hb |= 1u << u;
                    } else {
                        typename KeyWidth<KB>::Bucket w[U];
#pragma unroll
                        for (int u = 0; u < U; ++u)
                            w[u] = KeyWidth<KB>::load(keys + (size_t)(b[u] >> shift) * kBucketBytes,
                                                      q[u], S.empty_key);
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            bool any, open;
                            test_bucket(w[u], t[u], empty, any, open);
                            if (q[u] && (any || !open)) hb |= 1u << u;
                        }
                    }
                    hot |= (uint64_t)hb << (g - gs0);
                }
                for (; g < gs1; ++g) {  // tail: mark and resolve below
                    const K t = s ^ (KB == 32 ? (K)gk32[g].x : (K)gx64[g]);
                    if (sector(t)) hot |= 1ULL << (g - gs0);
                }
                while (hot) {
                    const int gc = gs0 + __ffsll((long long)hot) - 1;  // slot in shared memory
                    hot &= hot - 1ULL;
                    const int gr = t0 + gc;                             // index among the groups
                    const int gg = gr + (skip >= 0 && gr >= skip);
                    const uint64_t xv = __ldg(T.xmask + gg);
                    const uint32_t hxg = KB == 32 ? gk32[gc].y : gh64[gc];
                    const int m = lookup_hash_at<KB>(S, s64 ^ xv, (hs ^ hxg) >> shift, err);
                    if (m >= 0) acc.add(cmul(group_diag<R>(T, gg, s64), VT<V>::ld(x, m)));
                }
                __syncwarp();
            }
        }
        if (active) VT<V>::st(y, i, acc.get());
    }
}

// FM: the sector filter's form, chosen on the host from rq_subspace_t.fpoint (one kernel per
// form, so that the registers of the general bitset test do not weigh on the one-sector kernel)
template <typename V, int KB, int FM, int BLOCK, bool LF>
__global__ void __launch_bounds__(BLOCK, BLOCK == 1024 ? 1 : (sizeof(V) <= 8 ? 6 : 4))
k_matvec_hash(const rq_operator_t op, const V *__restrict__ x, V *__restrict__ y, int *err,
              const int *gate, const int *gate2) {
    constexpr int NB = KeyWidth<KB>::kNbytes;
    if (gate && (*gate == 0 || (gate2 && *gate2 == 0))) return;
    const rq_subspace_t &S = op.sub;
    const rq_terms_t &T = op.terms;
    init_hash_tables(hk_htab, NB);
    if (FM == kFiltSet)
        for (int w = threadIdx.x; w < RQ_FILTER_WORDS; w += blockDim.x) hk_fb[w] = S.fbits[w];
    __syncthreads();
    const int nres = T.J - (T.diag_group >= 0 ? 1 : 0);
    if (nres <= max_resident_groups<KB>())  // else in tiles
        load_group_keys<KB>(T, 0, nres, nres, S);
    __syncthreads();
    if (FM == kFiltPoint)
        hash_rows<V, KB, FM, LF, BLOCK == 1024>(op, x, y, err, S.fpoint / 65, S.fpoint % 65);
    else
        hash_rows<V, KB, FM, LF, BLOCK == 1024>(op, x, y, err, 0, 0);
}

// xhash[j] = h(xmask[j])
template <int KB>
__global__ void k_terms_hash(const uint64_t *__restrict__ xmask, int J, uint32_t *__restrict__ out) {
    __shared__ uint32_t htab[KeyWidth<KB>::kNbytes * 256];
    init_hash_tables(htab, KeyWidth<KB>::kNbytes);
    __syncthreads();
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < J; j += gridDim.x * blockDim.x)
        out[j] = lin_hash(htab, xmask[j], KeyWidth<KB>::kNbytes);
}

// ------------------------------------------------------------------------------------------
// FREE mode, generic lookups (sampled binary search; identity for the full space)
// ------------------------------------------------------------------------------------------
template <typename V, int LK>
__global__ void __launch_bounds__(kThreads)
k_matvec_free(const rq_operator_t op, const V *__restrict__ x, V *__restrict__ y, int gt, int kt,
              int stop_at_zero, int *err, const int *gate, const int *gate2) {
    using R = typename VT<V>::R;
    if (gate && (*gate == 0 || (gate2 && *gate2 == 0))) return;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_g1;
    const rq_subspace_t &S = op.sub;
    const rq_terms_t &T = op.terms;
    uint32_t *fb = reinterpret_cast<uint32_t *>(smem);
    uint64_t *samp = reinterpret_cast<uint64_t *>(smem + kFilterBytes);
    const int ns = (LK == RQ_LOOKUP_BSEARCH) ? (int)(S.D < kSample ? S.D : kSample) : 0;
    const Tile<R> tl =
        carve<R>(smem + kFilterBytes + (LK == RQ_LOOKUP_BSEARCH ? kSample * 8 : 0), gt, kt);
    load_lookup_smem<LK>(S, fb, samp, ns);

    const int64_t D = S.D;
    const bool d0 = (op.diag0 != nullptr) && (T.diag_group >= 0);
    const int gstart = (d0 && T.diag_group == 0) ? 1 : 0;
    const int skip = T.diag_group;  // handled outside the hit loop
    int g1_first = (gstart < T.J) ? load_tile<R>(T, gstart, gt, kt, tl, &s_g1) : T.J;
    if (g1_first < 0) {
        if (err && threadIdx.x == 0) atomicExch(err, RQ_E_RANGE);
        return;
    }
    __syncthreads();
    const bool resident = (g1_first >= T.J);
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < D;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const bool active = i < D;
        const uint64_t s =
            active ? (LK == RQ_LOOKUP_IDENTITY ? (uint64_t)i : __ldg(S.states + i)) : 0ULL;
        CAcc<R> acc;
        if (active && d0) {
            const R dv = (R)op.diag0[i];
            const cx<R> xv = VT<V>::ld(x, i);
            acc.add({dv * xv.re, dv * xv.im});
        }
        if (!resident && base != (int64_t)blockIdx.x * blockDim.x)
            g1_first = load_tile<R>(T, gstart, gt, kt, tl, &s_g1);
        int g0 = gstart, g1 = g1_first;
        while (g0 < T.J) {
            if (g1 < 0) {
                if (err && threadIdx.x == 0) atomicExch(err, RQ_E_RANGE);
                return;  // uniform across the block
            }
            if (active) {
                if (!d0 && skip >= g0 && skip < g1)
                    add_group<R>(tl.cf, tl.zm, tl.off[skip - g0], tl.off[skip - g0 + 1], s,
                                 VT<V>::ld(x, i), stop_at_zero, acc);
                for_hits<LK, 64>(S, fb, samp, ns, nullptr, tl.xm, g0, g1, skip, s, err,
                                 [&](int g, int64_t m) {
                                     add_group<R>(tl.cf, tl.zm, tl.off[g - g0], tl.off[g - g0 + 1],
                                                  s, VT<V>::ld(x, m), stop_at_zero, acc);
                                 });
            }
            if (g1 >= T.J) break;
            g0 = g1;
            g1 = load_tile<R>(T, g0, gt, kt, tl, &s_g1);
        }
        if (active) VT<V>::st(y, i, acc.get());
    }
}

// ------------------------------------------------------------------------------------------
// connectivity cache
// ------------------------------------------------------------------------------------------
template <int LK, int KB>
__global__ void __launch_bounds__(kThreads)
k_conn_count(const rq_operator_t op, int64_t *__restrict__ rowcnt, int *err) {
    __shared__ uint32_t fb[RQ_FILTER_WORDS];
    __shared__ uint64_t samp[LK == RQ_LOOKUP_BSEARCH ? kSample : 1];
    __shared__ uint32_t T[LK == RQ_LOOKUP_HASH ? kHashTableWords : 1];
    const rq_subspace_t &S = op.sub;
    const int ns = (LK == RQ_LOOKUP_BSEARCH) ? (int)(S.D < kSample ? S.D : kSample) : 0;
    load_lookup_smem<LK>(S, fb, samp, ns);
    if (LK == RQ_LOOKUP_HASH) init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.D;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = 0;
        for_hits<LK, KB>(S, fb, samp, ns, T, op.terms.xmask, 0, op.terms.J, op.terms.diag_group,
                         __ldg(S.states + i), err, [&](int, int64_t) { ++c; });
        rowcnt[i] = c;
    }
}

// Diagonal of group g for state s from the global term arrays (CONN mode and CSR values).


template <typename V, int LK, int KB>
__global__ void __launch_bounds__(kThreads)
k_conn_fill(const rq_operator_t op, const int64_t *__restrict__ rowptr, int32_t *__restrict__ col,
            int32_t *__restrict__ grp, V *__restrict__ val, int *err) {
    using R = typename VT<V>::R;
    __shared__ uint32_t fb[RQ_FILTER_WORDS];
    __shared__ uint64_t samp[LK == RQ_LOOKUP_BSEARCH ? kSample : 1];
    __shared__ uint32_t T[LK == RQ_LOOKUP_HASH ? kHashTableWords : 1];
    const rq_subspace_t &S = op.sub;
    const int ns = (LK == RQ_LOOKUP_BSEARCH) ? (int)(S.D < kSample ? S.D : kSample) : 0;
    load_lookup_smem<LK>(S, fb, samp, ns);
    if (LK == RQ_LOOKUP_HASH) init_hash_tables(T, KeyWidth<KB>::kNbytes);
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < S.D;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = rowptr[i];
        const uint64_t s = __ldg(S.states + i);
        for_hits<LK, KB>(S, fb, samp, ns, T, op.terms.xmask, 0, op.terms.J, op.terms.diag_group, s, err,
                     [&](int g, int64_t m) {
                         col[p] = (int32_t)m;
                         if (grp) grp[p] = g;
                         if (val) VT<V>::st(val, p, group_diag<R>(op.terms, g, s));
                         ++p;
                     });
    }
}

// Inclusive scan of rowptr[1..D] in place (three phases: block scans, scan of block totals,
// add block offsets).  Block b covers rows [b * 1024, (b + 1) * 1024).
__global__ void __launch_bounds__(kThreads) k_scan_blocks(int64_t *v, int64_t n, int64_t *bsum) {
    __shared__ int64_t ws[kThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * 1024;
    int64_t loc[4];
    int64_t t = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int64_t idx = base + threadIdx.x * 4 + k;
        loc[k] = (idx < n) ? v[idx] : 0;
        t += loc[k];
    }
    // exclusive scan of per-thread totals across the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t inc = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int64_t w = (lane < kThreads / 32) ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        if (lane < kThreads / 32) ws[lane] = w;
    }
    __syncthreads();
    int64_t run = inc - t + (warp > 0 ? ws[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int64_t idx = base + threadIdx.x * 4 + k;
        run += loc[k];
        if (idx < n) v[idx] = run;
    }
    if (threadIdx.x == kThreads - 1) bsum[blockIdx.x] = run;
}

__global__ void k_scan_totals(int64_t *bsum, int64_t nb) {
    // one block: sequential chunks per thread, then a block scan of chunk totals
    __shared__ int64_t tot[kThreads];
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t a = threadIdx.x * per, b = min(nb, a + per);
    int64_t s = 0;
    for (int64_t k = a; k < b; ++k) s += bsum[k];
    tot[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t r = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            const int64_t u = tot[k];
            tot[k] = r;
            r += u;
        }
    }
    __syncthreads();
    int64_t r = tot[threadIdx.x];
    for (int64_t k = a; k < b; ++k) {  // exclusive offsets of blocks
        const int64_t u = bsum[k];
        bsum[k] = r;
        r += u;
    }
}

__global__ void k_scan_add(int64_t *v, int64_t n, const int64_t *boff) {
    const int64_t base = (int64_t)blockIdx.x * 1024;
    const int64_t off = boff[blockIdx.x];
    for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
        const int64_t idx = base + k;
        if (idx < n) v[idx] += off;
    }
}

// ------------------------------------------------------------------------------------------
// CONN and CSR modes
// ------------------------------------------------------------------------------------------
template <typename V>
__global__ void __launch_bounds__(kThreads)
k_matvec_conn(const rq_operator_t op, const V *__restrict__ x, V *__restrict__ y, const int *gate,
              const int *gate2) {
    d_matvec_conn<V>(op, x, y, gate, gate2);
}

// VV: storage type of the element values (converted to the vector's precision on load)
template <typename V, typename VV>
__global__ void __launch_bounds__(kThreads)
k_matvec_csr(const rq_operator_t op, const V *__restrict__ x, V *__restrict__ y, const int *gate,
             const int *gate2) {
    d_matvec_csr<V, VV>(op, x, y, gate, gate2);
}

template <typename V>
int launch_csr(const rq_operator_t &op, const void *x, void *y, cudaStream_t st, const int *gate,
               const int *gate2, int grid) {
    const V *xx = static_cast<const V *>(x);
    V *yy = static_cast<V *>(y);
    switch (op.val_vtype) {
        case RQ_F32: k_matvec_csr<V, float><<<grid, kThreads, 0, st>>>(op, xx, yy, gate, gate2); break;
        case RQ_F64: k_matvec_csr<V, double><<<grid, kThreads, 0, st>>>(op, xx, yy, gate, gate2); break;
        case RQ_C64:
            if (!VT<V>::kComplex) return fail(RQ_E_ARG, "rq_matvec: complex CSR values need complex vectors");
            k_matvec_csr<V, float2><<<grid, kThreads, 0, st>>>(op, xx, yy, gate, gate2);
            break;
        case RQ_C128:
            if (!VT<V>::kComplex) return fail(RQ_E_ARG, "rq_matvec: complex CSR values need complex vectors");
            k_matvec_csr<V, double2><<<grid, kThreads, 0, st>>>(op, xx, yy, gate, gate2);
            break;
        default: return fail(RQ_E_ARG, "rq_matvec: bad val_vtype");
    }
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

// ------------------------------------------------------------------------------------------
// host dispatch
// ------------------------------------------------------------------------------------------
template <typename V, int KB, int FM, int BLOCK, bool LF>
int launch_hash_block(const rq_operator_t &op, const void *x, void *y, int *err, cudaStream_t st,
                      const int *gate, const int *gate2) {
    auto kern = k_matvec_hash<V, KB, FM, BLOCK, LF>;
    const int nres = op.terms.J - (op.terms.diag_group >= 0 ? 1 : 0);
    constexpr int kMaxRes = max_resident_groups<KB>();
    const size_t smem = group_key_bytes<KB>(nres < kMaxRes ? nres : kMaxRes);
    thread_local KernelLaunchCache table[kMaxCachedDevices];
    KernelLaunchCache *c = nullptr;
    int per_sm = 1;
    RQ_TRY(cache_slot(table, &c));
    RQ_TRY(configure_kernel(kern, *c, smem, BLOCK, &per_sm));
    int64_t g = (op.sub.D + BLOCK - 1) / BLOCK;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    if (g > cap) g = cap;
    kern<<<(int)(g < 1 ? 1 : g), BLOCK, smem, st>>>(op, static_cast<const V *>(x),
                                                   static_cast<V *>(y), err, gate, gate2);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

template <typename V, int KB, int FM>
int launch_hash(const rq_operator_t &op, const void *x, void *y, int *err, cudaStream_t st,
                const int *gate, const int *gate2) {
    // small group sets: several 256-thread blocks per SM; large ones (streamed in tiles of
    // max_resident_groups above that count): one 1024-thread block.
    // With a line filter the probes test its bits (not with 64-bit keys and the bitset filter,
    // whose line-filter kernel spills registers).
    const bool small = op.terms.J <= max_resident_groups<KB>() &&
                       group_key_bytes<KB>(op.terms.J) <= 16 * 1024;
    if (op.sub.lmap && !(KB == 64 && FM == kFiltSet))
        return small ? launch_hash_block<V, KB, FM, 256, true>(op, x, y, err, st, gate, gate2)
                     : launch_hash_block<V, KB, FM, 1024, true>(op, x, y, err, st, gate, gate2);
    return small ? launch_hash_block<V, KB, FM, 256, false>(op, x, y, err, st, gate, gate2)
                 : launch_hash_block<V, KB, FM, 1024, false>(op, x, y, err, st, gate, gate2);
}

template <typename V, int LK>
int launch_free(const rq_operator_t &op, const void *x, void *y, int stop_at_zero, int *err,
                cudaStream_t st, const int *gate = nullptr, const int *gate2 = nullptr) {
    using R = typename VT<V>::R;
    const rq_terms_t &T = op.terms;
    const int gt = T.J < kGT ? (T.J > 0 ? T.J : 1) : kGT;
    const int kt = T.K < kKT ? (T.K > 0 ? T.K : 1) : kKT;
    const size_t smem = kFilterBytes + (LK == RQ_LOOKUP_BSEARCH ? kSample * 8 : 0) +
                        tile_bytes<R>(gt, kt);
    auto kern = k_matvec_free<V, LK>;
    thread_local KernelLaunchCache table[kMaxCachedDevices];
    KernelLaunchCache *c = nullptr;
    int per_sm = 1;
    RQ_TRY(cache_slot(table, &c));
    RQ_TRY(configure_kernel(kern, *c, smem, kThreads, &per_sm));
    int64_t g = (op.sub.D + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    if (g > cap) g = cap;
    kern<<<(int)g, kThreads, smem, st>>>(op, static_cast<const V *>(x), static_cast<V *>(y), gt, kt,
                                         stop_at_zero, err, gate, gate2);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

int grid_rows(int64_t n) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * 8;
    return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

template <typename V>
int matvec_typed(const rq_operator_t &op, const void *x, void *y, void *scratch, cudaStream_t st,
                 const int *gate, const int *gate2) {
    int *err = scratch ? scratch_err(scratch) : nullptr;
    switch (op.mode) {
        case RQ_MODE_FREE:
            if (op.sub.lookup == RQ_LOOKUP_HASH) {
                // the sector filter is off when both masks are zero; a subspace in one sector
                // (fpoint >= 0) tests two popcounts instead of the bitset.  Behind a small line
                // filter the sector test costs more than it saves: a target it would reject
                // costs one L2-resident word of the line filter instead; a larger line filter
                // keeps it, since its words then compete for L2 or come from DRAM.
                const bool line_in_l2 =
                    op.sub.lmap && op.sub.lbits + op.sub.lwbits - 3 <= kLineFilterL2Log2Bytes;
                const int fm = ((op.sub.fmask_a | op.sub.fmask_b) == 0 || line_in_l2) ? kFiltNone
                               : op.sub.fpoint >= 0                                     ? kFiltPoint
                                                                                        : kFiltSet;
                if (op.sub.key_bits == 32) {
                    if (fm == kFiltPoint) return launch_hash<V, 32, kFiltPoint>(op, x, y, err, st, gate, gate2);
                    if (fm == kFiltSet) return launch_hash<V, 32, kFiltSet>(op, x, y, err, st, gate, gate2);
                    return launch_hash<V, 32, kFiltNone>(op, x, y, err, st, gate, gate2);
                }
                if (fm == kFiltPoint) return launch_hash<V, 64, kFiltPoint>(op, x, y, err, st, gate, gate2);
                if (fm == kFiltSet) return launch_hash<V, 64, kFiltSet>(op, x, y, err, st, gate, gate2);
                return launch_hash<V, 64, kFiltNone>(op, x, y, err, st, gate, gate2);
            }
            if (op.sub.lookup == RQ_LOOKUP_BSEARCH)
                return launch_free<V, RQ_LOOKUP_BSEARCH>(op, x, y, 1, err, st, gate, gate2);
            return fail(RQ_E_ARG, "rq_matvec: unsupported lookup for a subspace");
        case RQ_MODE_CONN:
            if (!op.rowptr || (op.nnz > 0 && (!op.col || !op.grp)))
                return fail(RQ_E_ARG, "rq_matvec: RQ_MODE_CONN needs rowptr, col and grp");
            k_matvec_conn<V><<<grid_rows(op.sub.D), kThreads, 0, st>>>(
                op, static_cast<const V *>(x), static_cast<V *>(y), gate, gate2);
            RQ_CUDA(cudaGetLastError());
            return RQ_OK;
        case RQ_MODE_CSR:
            if (!op.rowptr || (op.nnz > 0 && (!op.col || !op.val)))
                return fail(RQ_E_ARG, "rq_matvec: RQ_MODE_CSR needs rowptr, col and val");
            if (op.terms.diag_group >= 0 && !op.diag0)
                return fail(RQ_E_ARG, "rq_matvec: RQ_MODE_CSR needs diag0 when a diagonal group exists");
            return launch_csr<V>(op, x, y, st, gate, gate2, grid_rows(op.sub.D));
        default:
            return fail(RQ_E_ARG, "rq_matvec: unknown mode");
    }
}

int check_operator(const rq_operator_t *op, int32_t vtype) {
    if (!op) return fail(RQ_E_ARG, "null operator");
    const rq_terms_t &T = op->terms;
    if (T.J < 0 || T.K < 0 || (T.J > 0 && (!T.xmask || !T.toff)) || (T.K > 0 && (!T.zmask || !T.coef)))
        return fail(RQ_E_ARG, "terms: bad sizes or null arrays");
    if (T.diag_group >= T.J) return fail(RQ_E_ARG, "terms: diag_group out of range");
    if ((vtype == RQ_F32 || vtype == RQ_F64) && !T.is_real)
        return fail(RQ_E_ARG, "real vectors need real coefficients (terms.is_real)");
    if (vtype_size(vtype) == 0) return fail(RQ_E_ARG, "unknown value type");
    if (op->sub.D < 1 || op->sub.D >= (int64_t(1) << 31))
        return fail(RQ_E_RANGE, "subspace dimension must be in [1, 2^31)");
    return RQ_OK;
}

}  // namespace

// Inclusive scan of D row counts in place (block scans, scan of block totals, offsets).
int scan_row_counts(int64_t *v, int64_t D, int64_t *bsum, cudaStream_t st) {
    const int64_t nb = (D + 1023) / 1024;
    k_scan_blocks<<<(int)nb, kThreads, 0, st>>>(v, D, bsum);
    k_scan_totals<<<1, kThreads, 0, st>>>(bsum, nb);
    k_scan_add<<<(int)nb, kThreads, 0, st>>>(v, D, bsum);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

// entry used by the LOBPCG driver (same translation-unit-independent dispatch)
int matvec_dispatch(const rq_operator_t &op, int32_t vtype, const void *x, void *y, void *scratch,
                    cudaStream_t st, const int *gate, const int *gate2) {
    switch (vtype) {
        case RQ_F32: return matvec_typed<float>(op, x, y, scratch, st, gate, gate2);
        case RQ_F64: return matvec_typed<double>(op, x, y, scratch, st, gate, gate2);
        case RQ_C64: return matvec_typed<float2>(op, x, y, scratch, st, gate, gate2);
        case RQ_C128: return matvec_typed<double2>(op, x, y, scratch, st, gate, gate2);
        default: return fail(RQ_E_ARG, "unknown value type");
    }
}

}  // namespace rq

using namespace rq;

RQ_API int rq_matvec(const rq_operator_t *op, int32_t vtype, const void *x, void *y, void *scratch,
                     void *stream) {
    RQ_TRY(check_operator(op, vtype));
    if (!x || !y || x == y) return fail(RQ_E_ARG, "rq_matvec: x and y must be distinct non-null");
    if (op->mode == RQ_MODE_FREE && !scratch)
        return fail(RQ_E_ARG, "rq_matvec: RQ_MODE_FREE needs scratch (error flag)");
    return matvec_dispatch(*op, vtype, x, y, scratch, as_stream(stream), nullptr, nullptr);
}

RQ_API int rq_fullspace_matvec(const rq_terms_t *terms, int32_t n, int32_t vtype, const void *x,
                               void *y, void *stream) {
    if (!terms || !x || !y || x == y || n < 0 || n > 31)
        return fail(RQ_E_ARG, "rq_fullspace_matvec: bad arguments (n must be <= 31)");
    rq_operator_t op = {};
    op.terms = *terms;
    op.terms.diag_group = -1;  // the x = 0 group is handled like any other (source = row)
    op.sub.D = int64_t(1) << n;
    op.sub.lookup = RQ_LOOKUP_IDENTITY;
    op.mode = RQ_MODE_FREE;
    RQ_TRY(check_operator(&op, vtype));
    cudaStream_t st = as_stream(stream);
    // PauliSumXZ.matmul sums every stored coefficient (no stop at a zero), symplectic.py:142-147
    switch (vtype) {
        case RQ_F32: return launch_free<float, RQ_LOOKUP_IDENTITY>(op, x, y, 0, nullptr, st);
        case RQ_F64: return launch_free<double, RQ_LOOKUP_IDENTITY>(op, x, y, 0, nullptr, st);
        case RQ_C64: return launch_free<float2, RQ_LOOKUP_IDENTITY>(op, x, y, 0, nullptr, st);
        case RQ_C128: return launch_free<double2, RQ_LOOKUP_IDENTITY>(op, x, y, 0, nullptr, st);
        default: return fail(RQ_E_ARG, "unknown value type");
    }
}

RQ_API int rq_terms_hash(const rq_terms_t *terms, uint32_t *xhash, void *stream) {
    if (!terms || !xhash || terms->J < 0 || (terms->J > 0 && !terms->xmask))
        return fail(RQ_E_ARG, "rq_terms_hash: bad arguments");
    if (terms->J == 0) return RQ_OK;
    // the hash is GF(2)-linear over the key bytes; masks below 2^32 hash the same with the
    // 4-byte and the 8-byte tables, so the 8-byte tables serve both key widths
    const int grid = (terms->J + kThreads - 1) / kThreads;
    k_terms_hash<64><<<grid, kThreads, 0, as_stream(stream)>>>(terms->xmask, terms->J, xhash);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_terms_upload(int32_t J, int32_t K, const uint64_t *xmask, const int32_t *toff,
                           const uint64_t *zmask, const double *coef, uint64_t *d_xmask,
                           int32_t *d_toff, uint64_t *d_zmask, double *d_coef, uint32_t *d_xhash,
                           rq_terms_t *t, void *stream) {
    if (!t || J < 0 || K < 0 || !toff || !d_toff || (J > 0 && (!xmask || !d_xmask || !d_xhash)) ||
        (K > 0 && (!zmask || !coef || !d_zmask || !d_coef)))
        return fail(RQ_E_ARG, "rq_terms_upload: bad arguments");
    if (toff[0] != 0 || toff[J] != K) return fail(RQ_E_ARG, "rq_terms_upload: toff must span [0, K]");
    for (int32_t j = 0; j < J; ++j) {
        if (toff[j + 1] < toff[j]) return fail(RQ_E_ARG, "rq_terms_upload: toff decreases");
        if (j > 0 && xmask[j] <= xmask[j - 1])
            return fail(RQ_E_ARG, "rq_terms_upload: X masks must be strictly increasing");
    }
    int32_t real = 1;
    for (int64_t k = 0; k < K; ++k)
        if (coef[2 * k + 1] != 0.) real = 0;
    cudaStream_t st = as_stream(stream);
    if (J > 0) RQ_CUDA(cudaMemcpyAsync(d_xmask, xmask, sizeof(uint64_t) * J, cudaMemcpyHostToDevice, st));
    RQ_CUDA(cudaMemcpyAsync(d_toff, toff, sizeof(int32_t) * (J + 1), cudaMemcpyHostToDevice, st));
    if (K > 0) {
        RQ_CUDA(cudaMemcpyAsync(d_zmask, zmask, sizeof(uint64_t) * K, cudaMemcpyHostToDevice, st));
        RQ_CUDA(cudaMemcpyAsync(d_coef, coef, sizeof(double) * 2 * K, cudaMemcpyHostToDevice, st));
    }
    rq_terms_t T{};
    T.J = J;
    T.K = K;
    T.diag_group = (J > 0 && xmask[0] == 0) ? 0 : -1;
    T.is_real = real;
    T.xmask = d_xmask;
    T.toff = d_toff;
    T.zmask = d_zmask;
    T.coef = d_coef;
    T.xhash = nullptr;
    RQ_TRY(rq_terms_hash(&T, d_xhash, stream));
    T.xhash = J > 0 ? d_xhash : nullptr;
    RQ_CUDA(cudaStreamSynchronize(st));
    *t = T;
    return RQ_OK;
}

RQ_API int rq_conn_build(const rq_operator_t *op, int64_t *rowptr, int32_t *col, int32_t *grp,
                         void *val, int32_t vtype, int64_t *nnz, void *scratch, void *stream) {
    RQ_TRY(check_operator(op, val ? vtype : RQ_C128));
    if (!rowptr || !scratch || !nnz) return fail(RQ_E_ARG, "rq_conn_build: null argument");
    const rq_subspace_t &S = op->sub;
    if (S.lookup != RQ_LOOKUP_HASH && S.lookup != RQ_LOOKUP_BSEARCH)
        return fail(RQ_E_ARG, "rq_conn_build: needs a hash or binary-search subspace");
    cudaStream_t st = as_stream(stream);
    int *err = scratch_err(scratch);
    const int64_t D = S.D;
    if (!col) {
        RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        RQ_CUDA(cudaMemsetAsync(rowptr, 0, sizeof(int64_t), st));
        if (S.lookup == RQ_LOOKUP_HASH && S.key_bits == 32)
            k_conn_count<RQ_LOOKUP_HASH, 32><<<grid_rows(D), kThreads, 0, st>>>(*op, rowptr + 1, err);
        else if (S.lookup == RQ_LOOKUP_HASH)
            k_conn_count<RQ_LOOKUP_HASH, 64><<<grid_rows(D), kThreads, 0, st>>>(*op, rowptr + 1, err);
        else
            k_conn_count<RQ_LOOKUP_BSEARCH, 64><<<grid_rows(D), kThreads, 0, st>>>(*op, rowptr + 1, err);
        RQ_CUDA(cudaGetLastError());
        RQ_TRY(scan_row_counts(rowptr + 1, D, scratch_scan(scratch), st));
        int h_err = 0;
        RQ_CUDA(cudaMemcpyAsync(nnz, rowptr + D, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        if (h_err) return fail(h_err, "rq_conn_build: lookup failed");
        return RQ_OK;
    }
    const int g = grid_rows(D);
#define RQ_FILL(V)                                                                                  \
    do {                                                                                            \
        if (S.lookup == RQ_LOOKUP_HASH && S.key_bits == 32)                                         \
            k_conn_fill<V, RQ_LOOKUP_HASH, 32><<<g, kThreads, 0, st>>>(*op, rowptr, col, grp,       \
                                                                       static_cast<V *>(val), err); \
        else if (S.lookup == RQ_LOOKUP_HASH)                                                        \
            k_conn_fill<V, RQ_LOOKUP_HASH, 64><<<g, kThreads, 0, st>>>(*op, rowptr, col, grp,       \
                                                                       static_cast<V *>(val), err); \
        else                                                                                        \
            k_conn_fill<V, RQ_LOOKUP_BSEARCH, 64><<<g, kThreads, 0, st>>>(*op, rowptr, col, grp,    \
                                                                          static_cast<V *>(val), err); \
    } while (0)
    switch (val ? vtype : RQ_C128) {
        case RQ_F32: RQ_FILL(float); break;
        case RQ_F64: RQ_FILL(double); break;
        case RQ_C64: RQ_FILL(float2); break;
        case RQ_C128: RQ_FILL(double2); break;
        default: return fail(RQ_E_ARG, "rq_conn_build: unknown value type");
    }
#undef RQ_FILL
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}
