// Learned warm start: a BF16 MLP (64 -> 256 -> 256 -> 2, GELU) mapping (state, U) to the ground
// state's log-amplitude and sign, trained and evaluated with tcgen05 tensor-core GEMMs.
//
// GEMM: C[M][N] = A[M][K] B[N][K]^T, both operands K-major BF16, FP32 accumulators in TMEM.  A CTA
// of 128 threads owns a 128-row tile and all N <= 256 columns; K runs in chunks of 64 through a
// two-stage shared-memory ring filled with cp.async (16 B per thread and copy) in the no-swizzle
// core-matrix layout: an 8-row x 16-byte core matrix is 128 contiguous bytes, core matrices
// adjacent in K are 128 B apart (leading byte offset) and 8-row groups 1024 B apart (stride byte
// offset).  One thread issues four tcgen05.mma (K = 16 each) per chunk and commits them to the
// stage's mbarrier; the stage is refilled once that barrier completes, so the copies of chunk c
// overlap the MMAs of chunk c - 1.  The epilogue reads the accumulator rows back with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, one row per thread) and fuses bias, GELU,
// the 256 -> 2 output layer, GELU' and the bias-gradient column sums.
//
// Every mbarrier wait is bounded (about one second of clock cycles); on expiry the kernel records
// RQ_E_CUDA in the error flag, skips the remaining work, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kIn = RQ_MLP_IN, kHid = RQ_MLP_HIDDEN, kOut = RQ_MLP_OUT;
constexpr int kTileM = 128, kChunkK = 64;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kHid * kIn, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kOut * kHid,
              kNParams = kOffB3 + kOut;
static_assert(kNParams == RQ_MLP_NPARAMS, "parameter layout");
constexpr int kHeadPart = kHid + kOut * kHid + kOut;  // db2 | dW3 | db3 partial sums per tile
constexpr long long kWaitCycles = 2000000000LL;

enum Epi { EPI_F32 = 0, EPI_HIDDEN = 1, EPI_HEAD = 2, EPI_DGELU = 3, EPI_HEAD_TRAIN = 4 };

// ---------------------------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// bounded wait for the phase of the given parity; false when the limit expired (the abort flag is
// then set) or when another role has set the abort flag (abort may be null: no early exit)
__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, volatile int *abort) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (abort && *abort) return false;
        if (clock64() - t0 > kWaitCycles) {
            if (abort) *abort = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// 2-D TMA load of one box (x = column, y = row of the tensor map) into shared memory, completing
// on bar
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}
// barrier over nthreads threads returning the OR of their predicates (the same in every thread)
__device__ __forceinline__ bool named_bar_or(int id, int nthreads, bool p) {
    uint32_t r;
    asm volatile(
        "{\n.reg .pred pi, po;\nsetp.ne.b32 pi, %1, 0;\nbar.red.or.pred po, %2, %3, pi;\nselp.b32 %0, 1, 0, po;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)p), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// instruction descriptor of kind::f16: BF16 x BF16 -> FP32, both K-major, M x N
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
    return (1u << 4)                          // D: FP32
           | (1u << 7)                        // A: BF16
           | (1u << 10)                       // B: BF16
           | ((uint32_t)(N >> 3) << 17)       // N / 8
           | ((uint32_t)(M >> 4) << 24);      // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"  // in the same statement: the outputs exist after the wait
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// ---------------------------------------------------------------------------------------------
// activations
// ---------------------------------------------------------------------------------------------
// GELU in its tanh form (Hendrycks and Gimpel): 0.5 z (1 + tanh(k0 (z + k1 z^3))), k0 = sqrt(2 / pi),
// k1 = 0.044715, with the hardware tanh (tanh.approx.f32, relative error about 2^-11, below the BF16
// rounding of the activations): one special-function operation per element for the activation and
// its derivative together
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;\n" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluK0 = 0.7978845608028654f;           // sqrt(2 / pi)
constexpr float kGeluK01 = 0.7978845608028654f * 0.044715f;
__device__ __forceinline__ float gelu(float z) {
    return 0.5f * z * (1.f + tanh_approx(z * fmaf(kGeluK01, z * z, kGeluK0)));
}
// activation a and derivative d of one pre-activation
__device__ __forceinline__ void gelu_both(float z, float &a, float &d) {
    const float z2 = z * z;
    const float t = tanh_approx(z * fmaf(kGeluK01, z2, kGeluK0));
    const float h = 0.5f * (1.f + t);
    a = z * h;
    d = fmaf(0.5f * z * (1.f - t * t), fmaf(3.f * kGeluK01, z2, kGeluK0), h);
}
__device__ __forceinline__ float dgelu(float z) {
    float a, d;
    gelu_both(z, a, d);
    return d;
}

// ---------------------------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------------------------
constexpr int kGemmThreads = 320;  // warp 0: TMA producer, warp 1: MMA issuer, warps 2..9: epilogue
constexpr int kEpiThreads = 256;
constexpr int kEpiBar = 1;         // named barrier of the epilogue warps (0 is __syncthreads)
constexpr uint32_t kTileABytes = kTileM * kChunkK * 2;
constexpr int kSplitK = 76;        // K splits of the row-reduction GEMMs (2 row tiles x 76 = 152 units)

struct GemmArgs {
    int64_t M;        // rows of A; rows >= M are read as zeros (TMA fill) and not stored
    int64_t mtiles;   // ceil(M / 128)
    int64_t nsplit;   // K splits; EPI_F32 writes one partial product per split
    int64_t nchunks;  // K / 64
    const float *bias;
    bf16 *z_rm;       // pre-activations, row-major [M][N] (HIDDEN, HEAD; optional)
    bf16 *h_rm;       // activations, row-major [M][N] (HIDDEN)
    bf16 *h_fm;       // feature-major [N][ld_fm]: HIDDEN activations (optional), DGELU and HEAD_TRAIN gradients
    int64_t ld_fm;
    const bf16 *zin_rm;  // pre-activations read by DGELU, row-major [M][N]
    float *out;          // F32: [M][N], or [nsplit][N][M] with split_cm; HEAD, HEAD_TRAIN: [M][2] (optional)
    int split_cm;        // F32: column-major partial products (lane = row: coalesced stores)
    const float *w3;     // HEAD, HEAD_TRAIN: [2][N]
    const float *b3;     // HEAD, HEAD_TRAIN: [2]
    const float *tgt;    // HEAD_TRAIN: [M][3] = log-amplitude target, sign, weight
    float inv_rows;      // HEAD_TRAIN: 1 / rows (the loss is a mean over the rows)
    bf16 *dz_rm;         // HEAD_TRAIN: dZ2, row-major [M][N]
    float *colpart;      // DGELU: [gridDim.x][N]; HEAD_TRAIN: [gridDim.x][kHeadPart] (one row per CTA)
    double *losspart;    // HEAD_TRAIN: [gridDim.x]
    int *err;
};

template <int N, bool BRES>
struct GemmCfg {
    static constexpr uint32_t kBChunk = (uint32_t)N * kChunkK * 2;  // one 64-wide K chunk of B
    static constexpr int kStages = BRES ? 4 : (N == 256 ? 4 : 8);
    static constexpr uint32_t kStageBytes = kTileABytes + (BRES ? 0u : kBChunk);
};

// epilogue constants in shared memory: bias | W3 row 0 | W3 row 1
template <int N, int EPI>
__host__ __device__ constexpr int const_floats() {
    return EPI == EPI_HIDDEN ? N : ((EPI == EPI_HEAD || EPI == EPI_HEAD_TRAIN) ? 3 * N : 4);
}
// column sums accumulated per CTA: DGELU db1; HEAD_TRAIN db2, dW3 row 0, dW3 row 1
template <int EPI>
__host__ __device__ constexpr int colsum_quantities() {
    return EPI == EPI_HEAD_TRAIN ? 3 : (EPI == EPI_DGELU ? 1 : 0);
}

// lane l returns sum over the 32 lanes of v[l] (v is consumed): each of the five exchange rounds
// halves the columns a lane keeps, 31 shuffles for 32 column sums, in a fixed order
__device__ __forceinline__ float col_sum32(float (&v)[32], int lane) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float send = up ? v[i] : v[i + o];
            const float keep = up ? v[i + o] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ void store_bf16x32(bf16 *dst, const float (&v)[32]) {
    __align__(16) bf16 b[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) b[i] = __float2bfloat16_rn(v[i]);
#pragma unroll
    for (int i = 0; i < 4; ++i) reinterpret_cast<uint4 *>(dst)[i] = reinterpret_cast<const uint4 *>(b)[i];
}

// 32 consecutive floats of shared memory (16-byte aligned; the same address in every lane)
__device__ __forceinline__ void lds32(const float *p, float (&v)[32]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float4 t = reinterpret_cast<const float4 *>(p)[i];
        v[4 * i] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

// running sums of the epilogue over the CTA's tiles: col points at this thread's row quarter of the
// shared array csum[quantity][quarter][N] (quantity j at col[4 N j + c]; each (quarter, column) slot
// belongs to one thread); d0, d1 and loss per thread
template <int N, int EPI>
struct EpiAcc {
    float *col;
    float d0 = 0.f, d1 = 0.f;
    double loss = 0.;
};

// one epilogue thread: row `row` of the tile (its TMEM lane), columns [h N/2, (h + 1) N/2)
template <int N, int EPI>
__device__ __forceinline__ void epilogue(const GemmArgs &g, uint32_t taddr, int h, int lane, int row, int64_t m,
                                         bool valid, int64_t sp, int par, float (*xch)[kTileM][2],
                                         const float *cst, EpiAcc<N, EPI> &acc) {
    constexpr int kHalf = N / 2;
    const int col0 = h * kHalf;
    if constexpr (EPI == EPI_F32) {
#pragma unroll 1
        for (int g0 = 0; g0 < kHalf; g0 += 32) {
            float v[32];
            tmem_ld32(taddr + (uint32_t)(col0 + g0), v);
            if (valid) {
                if (g.split_cm) {
                    float *dst = g.out + (sp * N + col0 + g0) * g.M + m;
#pragma unroll
                    for (int i = 0; i < 32; ++i) dst[(int64_t)i * g.M] = v[i];
                } else {
                    float4 *dst = reinterpret_cast<float4 *>(g.out + m * N + col0 + g0);
#pragma unroll
                    for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
                }
            }
        }
    } else if constexpr (EPI == EPI_HIDDEN) {
#pragma unroll 1
        for (int g0 = 0; g0 < kHalf; g0 += 32) {
            const int c0 = col0 + g0;
            float z[32], b[32];
            tmem_ld32(taddr + (uint32_t)c0, z);
            lds32(cst + c0, b);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                z[i] += b[i];
                b[i] = gelu(z[i]);
            }
            if (valid) {
                if (g.z_rm) store_bf16x32(g.z_rm + m * N + c0, z);
                store_bf16x32(g.h_rm + m * N + c0, b);
                if (g.h_fm) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) g.h_fm[(int64_t)(c0 + i) * g.ld_fm + m] = __float2bfloat16_rn(b[i]);
                }
            }
        }
    } else if constexpr (EPI == EPI_HEAD || EPI == EPI_HEAD_TRAIN) {
        // pass 1: Z2 = acc + b2, H2 = GELU(Z2), the output layer's dot products over this half
        float o0 = 0.f, o1 = 0.f;
#pragma unroll 1
        for (int g0 = 0; g0 < kHalf; g0 += 32) {
            const int c0 = col0 + g0;
            float z[32], w[32];
            tmem_ld32(taddr + (uint32_t)c0, z);
            lds32(cst + c0, w);
#pragma unroll
            for (int i = 0; i < 32; ++i) z[i] += w[i];
            if (EPI == EPI_HEAD && valid && g.z_rm) store_bf16x32(g.z_rm + m * N + c0, z);
#pragma unroll
            for (int i = 0; i < 32; ++i) z[i] = gelu(z[i]);
            lds32(cst + N + c0, w);
#pragma unroll
            for (int i = 0; i < 32; ++i) o0 += z[i] * w[i];
            lds32(cst + 2 * N + c0, w);
#pragma unroll
            for (int i = 0; i < 32; ++i) o1 += z[i] * w[i];
        }
        if (h == 1) {
            xch[par][row][0] = o0;
            xch[par][row][1] = o1;
        }
        named_bar_sync(kEpiBar, kEpiThreads);
        if (h == 0) {
            o0 += xch[par][row][0] + __ldg(g.b3);
            o1 += xch[par][row][1] + __ldg(g.b3 + 1);
            if (valid && g.out) {
                g.out[m * 2] = o0;
                g.out[m * 2 + 1] = o1;
            }
        }
        if constexpr (EPI == EPI_HEAD_TRAIN) {
            // the loss of the row and its gradient (half 0), handed to half 1 through xch[par + 2]
            float d0 = 0.f, d1 = 0.f;
            if (h == 0) {
                if (valid) {
                    const float at = g.tgt[m * 3], sg = g.tgt[m * 3 + 1], w = g.tgt[m * 3 + 2];
                    const float e = o0 - at;
                    const float tt = -sg * o1;
                    const float sp = tt > 20.f ? tt : log1pf(expf(tt));  // softplus(-s o1)
                    const float sig = 1.f / (1.f + expf(-tt));           // sigmoid(-s o1)
                    acc.loss += (double)(w * (e * e + sp));
                    d0 = w * g.inv_rows * 2.f * e;
                    d1 = -w * g.inv_rows * sg * sig;
                }
                acc.d0 += d0;
                acc.d1 += d1;
                xch[par + 2][row][0] = d0;
                xch[par + 2][row][1] = d1;
            }
            named_bar_sync(kEpiBar, kEpiThreads);
            if (h == 1) {
                d0 = xch[par + 2][row][0];
                d1 = xch[par + 2][row][1];
            }
            // pass 2: dZ2 = (dout W3) * GELU'(Z2) and the column sums of db2 and dW3
#pragma unroll 1
            for (int g0 = 0; g0 < kHalf; g0 += 32) {
                const int c0 = col0 + g0;
                float z[32], a[32], t[32];
                tmem_ld32(taddr + (uint32_t)c0, z);
                lds32(cst + c0, t);
#pragma unroll
                for (int i = 0; i < 32; ++i) gelu_both(z[i] + t[i], a[i], z[i]);
                lds32(cst + N + c0, t);
#pragma unroll
                for (int i = 0; i < 32; ++i) t[i] *= d0;
                {
                    float w1[32];
                    lds32(cst + 2 * N + c0, w1);
#pragma unroll
                    for (int i = 0; i < 32; ++i) z[i] *= fmaf(d1, w1[i], t[i]);
                }
                if (valid) {
                    store_bf16x32(g.dz_rm + m * N + c0, z);
#pragma unroll
                    for (int i = 0; i < 32; ++i) g.h_fm[(int64_t)(c0 + i) * g.ld_fm + m] = __float2bfloat16_rn(z[i]);
                }
                float *cs = acc.col + c0 + lane;  // this thread's running sums, one column each
                cs[0] += col_sum32(z, lane);
#pragma unroll
                for (int i = 0; i < 32; ++i) t[i] = d0 * a[i];
                cs[4 * N] += col_sum32(t, lane);
#pragma unroll
                for (int i = 0; i < 32; ++i) t[i] = d1 * a[i];
                cs[8 * N] += col_sum32(t, lane);
            }
        }
    } else {  // EPI_DGELU: dZ1 = acc * GELU'(Z1), feature-major, with the column sums of db1
#pragma unroll 1
        for (int g0 = 0; g0 < kHalf; g0 += 32) {
            const int c0 = col0 + g0;
            float v[32];
            tmem_ld32(taddr + (uint32_t)c0, v);
            __align__(16) bf16 zin[32];
            if (valid) {
                const uint4 *src = reinterpret_cast<const uint4 *>(g.zin_rm + m * N + c0);
#pragma unroll
                for (int i = 0; i < 4; ++i) reinterpret_cast<uint4 *>(zin)[i] = src[i];
            }
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] = valid ? v[i] * dgelu(__bfloat162float(zin[i])) : 0.f;
            if (valid) {
#pragma unroll
                for (int i = 0; i < 32; ++i) g.h_fm[(int64_t)(c0 + i) * g.ld_fm + m] = __float2bfloat16_rn(v[i]);
            }
            acc.col[c0 + lane] += col_sum32(v, lane);
        }
    }
}

// shared-memory matrix descriptor of a K-major operand in the 128-byte swizzled layout that a TMA
// load with CU_TENSOR_MAP_SWIZZLE_128B writes to a 1 KB-aligned tile (rows of 128 B = 64 BF16 of K,
// 8-row atoms of 1 KB in which row r's 16-byte chunks are permuted by r mod 8): stride byte offset
// 1024 between 8-row groups, leading byte offset unused (one MMA's 16-wide K slice lies within a
// row), and the K slice kk of a 64-wide chunk starts 32 kk bytes into the tile (the hardware
// applies the permutation to the address)
__device__ __forceinline__ uint64_t make_sdesc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;               // leading byte offset, unused
    d |= (uint64_t)(1024u >> 4) << 32;    // stride byte offset
    d |= (uint64_t)1 << 46;               // descriptor version of tcgen05
    d |= (uint64_t)2 << 61;               // swizzle mode: 128 B
    return d;
}

// C = A B^T over the units (row tile, K split) of the grid-stride loop.  BRES: B (N x K, K <= 256)
// is loaded once and stays in shared memory; otherwise each stage of the ring holds a 64-wide K
// chunk of A and of B.  Every operand tile is one TMA box of 64 columns (128 B) x its rows.
template <int N, int EPI, bool BRES>
__global__ void __launch_bounds__(kGemmThreads, 1)
k_gemm(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b, const GemmArgs g) {
    static_assert(N == 64 || N == 256, "N is 64 or 256");
    using C = GemmCfg<N, BRES>;
    constexpr int S = C::kStages;
    constexpr int kNQ = colsum_quantities<EPI>();
    constexpr uint32_t kIdesc = make_idesc(kTileM, N);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2], bfull, fin;
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s, bwait_s;
    __shared__ long long issued_s, consumed_s;
    __shared__ __align__(16) float cst[const_floats<N, EPI>()];
    __shared__ float xch[(EPI == EPI_HEAD || EPI == EPI_HEAD_TRAIN) ? 4 : 1][kTileM][2];
    __shared__ float csum[kNQ > 0 ? kNQ : 1][4][kNQ > 0 ? N : 1];
    __shared__ float dsum[4][2];
    __shared__ double lsum[4];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t units = g.mtiles * g.nsplit;
    const uint32_t sbase = (smem_u32(smem) + 1023u) & ~1023u;  // the launch adds 1 KB for this
    const uint32_t ring = BRES ? (uint32_t)g.nchunks * C::kBChunk : 0u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpiThreads / 32);
        }
        mbar_init(&bfull, 1);
        mbar_init(&fin, 1);
        fence_mbar_init();
        abort_s = 0;
        bwait_s = 0;
        issued_s = 0;
        consumed_s = 0;
    }
    if (warp == 1) tmem_alloc(&tmem_s, 2u * N);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_s;
    volatile int *abort_p = &abort_s;

    if (warp == 0) {  // ---- TMA producer
        if (BRES && lane == 0) {
            mbar_expect_tx(&bfull, (uint32_t)g.nchunks * C::kBChunk);
            for (int c = 0; c < (int)g.nchunks; ++c)
                tma_load_2d(sbase + (uint32_t)c * C::kBChunk, &tma_b, c * kChunkK, 0, &bfull);
        }
        long long it = 0;
        bool bad = false;
        for (int64_t u = blockIdx.x; u < units && !bad; u += gridDim.x) {
            const int64_t mt = u % g.mtiles, sp = u / g.mtiles;
            const int64_t c0 = sp * g.nchunks / g.nsplit, c1 = (sp + 1) * g.nchunks / g.nsplit;
            for (int64_t c = c0; c < c1; ++c, ++it) {
                const int s = (int)(it % S);
                if (it >= S && !wait_bar(&empty[s], (uint32_t)((it / S - 1) & 1), abort_p)) {
                    bad = true;
                    break;
                }
                if (lane == 0) {
                    const uint32_t st = sbase + ring + (uint32_t)s * C::kStageBytes;
                    mbar_expect_tx(&full[s], C::kStageBytes);
                    tma_load_2d(st, &tma_a, (int)(c * kChunkK), (int)(mt * kTileM), &full[s]);
                    if (!BRES) tma_load_2d(st + kTileABytes, &tma_b, (int)(c * kChunkK), 0, &full[s]);
                    issued_s = it + 1;
                }
                __syncwarp();
            }
        }
    } else if (warp == 1) {  // ---- MMA issuer
        bool bad = BRES && !wait_bar(&bfull, 0u, abort_p);
        if (BRES && !bad && lane == 0) bwait_s = 1;
        long long it = 0, t = 0;
        for (int64_t u = blockIdx.x; u < units && !bad; u += gridDim.x, ++t) {
            const int b = (int)(t & 1);
            if (t >= 2 && !wait_bar(&tempty[b], (uint32_t)((t / 2 - 1) & 1), abort_p)) break;
            tc_fence_after();
            const int64_t sp = u / g.mtiles;
            const int64_t c0 = sp * g.nchunks / g.nsplit, c1 = (sp + 1) * g.nchunks / g.nsplit;
            const uint32_t acc = tmem + (uint32_t)(b * N);
            for (int64_t c = c0; c < c1; ++c, ++it) {
                const int s = (int)(it % S);
                if (!wait_bar(&full[s], (uint32_t)((it / S) & 1), abort_p)) {
                    bad = true;
                    break;
                }
                tc_fence_after();
                if (lane == 0) {
                    const uint32_t sa = sbase + ring + (uint32_t)s * C::kStageBytes;
                    const uint32_t sb = BRES ? sbase + (uint32_t)c * C::kBChunk : sa + kTileABytes;
#pragma unroll
                    for (int kk = 0; kk < kChunkK / 16; ++kk)
                        mma_bf16(acc, make_sdesc_sw128(sa + (uint32_t)kk * 32u), make_sdesc_sw128(sb + (uint32_t)kk * 32u),
                                 kIdesc, (c > c0 || kk > 0) ? 1u : 0u);
                    mma_commit(&empty[s]);
                    consumed_s = it + 1;
                }
                __syncwarp();
            }
            if (bad) break;
            if (lane == 0) mma_commit(&tfull[b]);
            __syncwarp();
        }
    } else {  // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 and half (w - 2) / 4 of the columns
        const int q = warp & 3, h = (warp - 2) >> 2, row = 32 * q + lane, e = threadIdx.x - 64;
        if constexpr (const_floats<N, EPI>() > 4) {
            for (int i = e; i < N; i += kEpiThreads) {
                cst[i] = g.bias[i];
                if (EPI != EPI_HIDDEN) {
                    cst[N + i] = g.w3[i];
                    cst[2 * N + i] = g.w3[N + i];
                }
            }
            named_bar_sync(kEpiBar, kEpiThreads);
        }
        EpiAcc<N, EPI> acc;
        acc.col = &csum[0][q][0];
        if constexpr (kNQ > 0) {
            for (int j = 0; j < kNQ; ++j)
                for (int k = 0; k < N / 64; ++k) csum[j][q][h * (N / 2) + 32 * k + lane] = 0.f;
        }
        bool broke = false;
        long long t = 0;
        for (int64_t u = blockIdx.x; u < units; u += gridDim.x, ++t) {
            const int b = (int)(t & 1);
            const bool ok = wait_bar(&tfull[b], (uint32_t)((t >> 1) & 1), abort_p);
            if (named_bar_or(kEpiBar, kEpiThreads, !ok || *abort_p != 0)) {  // the same answer in every epilogue thread
                broke = true;
                break;
            }
            tc_fence_after();
            const int64_t mt = u % g.mtiles, sp = u / g.mtiles;
            const int64_t m = mt * kTileM + row;
            epilogue<N, EPI>(g, tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * N), h, lane, row, m, m < g.M, sp,
                             b, xch, cst, acc);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
        if (kNQ > 0 && !broke) {
            // this CTA's column sums: the four row quarters added in order, one row of partials
            if (EPI == EPI_HEAD_TRAIN && h == 0) {
                const float s0 = warp_sum(acc.d0), s1 = warp_sum(acc.d1);
                const double sl = warp_sum(acc.loss);
                if (lane == 0) {
                    dsum[q][0] = s0;
                    dsum[q][1] = s1;
                    lsum[q] = sl;
                }
            }
            named_bar_sync(kEpiBar, kEpiThreads);
            float *part = g.colpart + (int64_t)blockIdx.x * (EPI == EPI_HEAD_TRAIN ? kHeadPart : N);
            for (int c = e; c < N; c += kEpiThreads)
#pragma unroll
                for (int j = 0; j < (kNQ > 0 ? kNQ : 1); ++j)
                    part[j * N + c] = ((csum[j][0][c] + csum[j][1][c]) + csum[j][2][c]) + csum[j][3][c];
            if (EPI == EPI_HEAD_TRAIN && e == 0) {
                part[3 * N] = ((dsum[0][0] + dsum[1][0]) + dsum[2][0]) + dsum[3][0];
                part[3 * N + 1] = ((dsum[0][1] + dsum[1][1]) + dsum[2][1]) + dsum[3][1];
                g.losspart[blockIdx.x] = ((lsum[0] + lsum[1]) + lsum[2]) + lsum[3];
            }
        }
    }
    __syncthreads();
    const bool aborted = abort_s != 0;
    if (aborted) {
        // let the copies and MMAs already issued land before the memory is released
        if (threadIdx.x == 0) {
            for (long long it = consumed_s; it < issued_s; ++it) {
                const int s = (int)(it % S);
                wait_bar(&full[s], (uint32_t)((it / S) & 1), nullptr);
            }
            if (BRES && !bwait_s) wait_bar(&bfull, 0u, nullptr);
            if (g.err) atomicExch(g.err, RQ_E_CUDA);
        }
        if (warp == 1) {
            if (lane == 0) mma_commit(&fin);
            __syncwarp();
            wait_bar(&fin, 0u, nullptr);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 2u * N);
    }
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiledFn *out) {
    static std::atomic<void *> cached{nullptr};
    void *p = cached.load();
    if (!p) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        RQ_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) return fail(RQ_E_CUDA, "cuTensorMapEncodeTiled not available");
        cached.store(p);
    }
    *out = reinterpret_cast<EncodeTiledFn>(p);
    return RQ_OK;
}

// BF16 matrix of `rows` rows x `cols` columns (row stride ld elements, cols a multiple of 64) read
// in boxes of 64 columns x box_rows rows with the 128-byte swizzle; rows past the end read as zeros
int make_tma(CUtensorMap *map, const bf16 *base, int64_t cols, int64_t rows, int64_t ld, int box_rows) {
    if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || ld % 8 != 0 || cols % kChunkK != 0)
        return fail(RQ_E_ARG, "bf16 GEMM: operands need 16-byte aligned rows");
    EncodeTiledFn enc = nullptr;
    RQ_TRY(encode_fn(&enc));
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16 *>(base), dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(RQ_E_CUDA, "cuTensorMapEncodeTiled failed");
    return RQ_OK;
}

// A [M][K] (lda), B [N][K] (ldb), K a multiple of 64; g.M, g.nsplit and the epilogue fields set by
// the caller; *grid_out (optional) = the CTAs launched (rows of the per-CTA partial sums)
template <int N, int EPI, bool BRES>
int launch_gemm_t(const bf16 *A, int64_t lda, const bf16 *B, int64_t ldb, int64_t K, GemmArgs g, cudaStream_t st,
                  int64_t *grid_out) {
    using C = GemmCfg<N, BRES>;
    if (g.M < 1 || K < kChunkK || K % kChunkK != 0 || g.nsplit < 1 || g.nsplit > K / kChunkK || (BRES && K > 256))
        return fail(RQ_E_ARG, "bf16 GEMM: bad shape");
    g.mtiles = (g.M + kTileM - 1) / kTileM;
    g.nchunks = K / kChunkK;
    CUtensorMap ta, tb;
    RQ_TRY(make_tma(&ta, A, K, g.M, lda, kTileM));
    RQ_TRY(make_tma(&tb, B, K, N, ldb, N));
    uint32_t smem = BRES ? (uint32_t)g.nchunks * C::kBChunk + C::kStages * kTileABytes : C::kStages * C::kStageBytes;
    smem += 1024;  // alignment of the operand tiles to 1 KB
    if (N == 256 && smem < 116u * 1024u) smem = 116u * 1024u;  // one CTA per SM: its 512 TMEM columns are all of them
    thread_local KernelLaunchCache table[kMaxCachedDevices];
    KernelLaunchCache *c = nullptr;
    int per_sm = 1;
    RQ_TRY(cache_slot(table, &c));
    RQ_TRY(configure_kernel(k_gemm<N, EPI, BRES>, *c, smem, kGemmThreads, &per_sm));
    const int64_t units = g.mtiles * g.nsplit;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    const int64_t grid = units < cap ? units : cap;
    if (grid > 0x7FFFFFFF) return fail(RQ_E_RANGE, "bf16 GEMM: grid out of range");
    k_gemm<N, EPI, BRES><<<(unsigned)grid, kGemmThreads, smem, st>>>(ta, tb, g);
    RQ_CUDA(cudaGetLastError());
    if (grid_out) *grid_out = grid;
    return RQ_OK;
}

template <int N, int EPI>
int launch_gemm(const bf16 *A, int64_t lda, const bf16 *B, int64_t ldb, int64_t K, const GemmArgs &g,
                cudaStream_t st, int64_t *grid_out = nullptr) {
    if constexpr (EPI == EPI_F32) {  // K <= 256: B stays in shared memory; else B streams with A
        if (K <= 256 && g.nsplit == 1) return launch_gemm_t<N, EPI, true>(A, lda, B, ldb, K, g, st, grid_out);
        return launch_gemm_t<N, EPI, false>(A, lda, B, ldb, K, g, st, grid_out);
    } else {  // the layer GEMMs: K = 64 or 256
        return launch_gemm_t<N, EPI, true>(A, lda, B, ldb, K, g, st, grid_out);
    }
}

// ---------------------------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float feature(uint64_t s, double u, int f) {
    if (f < 32) return ((s >> f) & 1ULL) ? 1.f : -1.f;
    if (f == 32) return (float)u;
    if (f == 33) return (float)(u * u);
    if (f == 34) return (float)(u * u * u);
    return 0.f;
}

__device__ __forceinline__ void write_features(bf16 *row, uint64_t s, double u) {
#pragma unroll
    for (int f0 = 0; f0 < kIn; f0 += 8) {
        __align__(16) bf16 b[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) b[q] = __float2bfloat16_rn(feature(s, u, f0 + q));
        *reinterpret_cast<uint4 *>(row + f0) = *reinterpret_cast<const uint4 *>(b);
    }
}

__global__ void k_features(const uint64_t *__restrict__ S, int64_t D, double U, bf16 *__restrict__ x) {
    const double u = (U - 5.0) / 3.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D; k += (int64_t)gridDim.x * blockDim.x)
        write_features(x + k * kIn, S[k], u);
}

__global__ void k_sample(const uint64_t *__restrict__ S, int64_t D, const double *__restrict__ U,
                         const float *__restrict__ psi, int P, uint64_t seed, int64_t step, int64_t rows,
                         bf16 *__restrict__ x, bf16 *__restrict__ xt, float *__restrict__ tgt) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < rows; m += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t r = mix64(seed ^ mix64((uint64_t)step * 0x100000001B3ULL + (uint64_t)m));
        const int i = (int)((r >> 32) % (uint64_t)P);
        const int64_t k = (int64_t)((r & 0xFFFFFFFFULL) % (uint64_t)D);
        const uint64_t s = S[k];
        const double u = (U[i] - 5.0) / 3.0;
        write_features(x + m * kIn, s, u);
        for (int f = 0; f < kIn; ++f) xt[(int64_t)f * rows + m] = __float2bfloat16_rn(feature(s, u, f));
        const float p = psi[(int64_t)i * D + k];
        const float ap = fabsf(p);
        const float a = logf(fmaxf(ap, 1e-30f)) + 0.5f * logf((float)D);
        const float w = fminf(fmaxf((float)D * p * p, 0.05f), 20.f);
        tgt[m * 3] = fmaxf(a, -30.f);
        tgt[m * 3 + 1] = p < 0.f ? -1.f : 1.f;
        tgt[m * 3 + 2] = w;
    }
}

// loss and its gradient; one partial sum per block (summed in block order by k_loss_sum)
__global__ void k_loss(int64_t rows, const float *__restrict__ out, const float *__restrict__ tgt,
                       float *__restrict__ dout, double *__restrict__ part) {
    __shared__ double red[kThreads / 32];
    const float inv = 1.f / (float)rows;
    double acc = 0.;
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < rows; m += (int64_t)gridDim.x * blockDim.x) {
        const float o0 = out[m * 2], o1 = out[m * 2 + 1];
        const float a = tgt[m * 3], sg = tgt[m * 3 + 1], w = tgt[m * 3 + 2];
        const float e = o0 - a;
        const float t = -sg * o1;
        const float sp = t > 20.f ? t : log1pf(expf(t));  // softplus(-s o1)
        const float sig = 1.f / (1.f + expf(-t));         // sigmoid(-s o1)
        acc += (double)(w * (e * e + sp));
        dout[m * 2] = w * inv * 2.f * e;
        dout[m * 2 + 1] = -w * inv * sg * sig;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        part[blockIdx.x] = s;
    }
}

// loss = sum of the n partial sums / rows: thread t adds part[t], part[t + 256], ... in order, then
// a fixed tree over the threads (the same sum on every run)
__global__ void __launch_bounds__(kThreads) k_loss_sum(const double *__restrict__ part, int n, int64_t rows,
                                                       double *loss) {
    __shared__ double red[kThreads];
    double s = 0.;
    for (int i = threadIdx.x; i < n; i += kThreads) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (double)rows;
}

// backward through the output layer: thread j = hidden unit j, 128 rows per block
__global__ void __launch_bounds__(kHid) k_head_bwd(const bf16 *__restrict__ z2, const float *__restrict__ dout,
                                                   const float *__restrict__ params, int64_t rows,
                                                   bf16 *__restrict__ dz2_rm, bf16 *__restrict__ dz2_fm,
                                                   float *__restrict__ part) {
    __shared__ float d_s[kTileM][2];
    const int64_t m0 = (int64_t)blockIdx.x * kTileM;
    for (int i = threadIdx.x; i < kTileM * 2; i += blockDim.x) d_s[i >> 1][i & 1] = dout[m0 * 2 + i];
    __syncthreads();
    const int j = threadIdx.x;
    const float w30 = params[kOffW3 + j], w31 = params[kOffW3 + kHid + j];
    float aw0 = 0.f, aw1 = 0.f, ab = 0.f;
    for (int r0 = 0; r0 < kTileM; r0 += 8) {
        __align__(16) bf16 buf[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int64_t m = m0 + r0 + q;
            const float z = __bfloat162float(z2[m * kHid + j]);
            const float h = gelu(z);
            const float d0 = d_s[r0 + q][0], d1 = d_s[r0 + q][1];
            const float dz = (d0 * w30 + d1 * w31) * dgelu(z);
            const bf16 b = __float2bfloat16_rn(dz);
            dz2_rm[m * kHid + j] = b;
            buf[q] = b;
            aw0 += d0 * h;
            aw1 += d1 * h;
            ab += dz;
        }
        *reinterpret_cast<uint4 *>(dz2_fm + (int64_t)j * rows + m0 + r0) = *reinterpret_cast<const uint4 *>(buf);
    }
    float *p = part + (int64_t)blockIdx.x * kHeadPart;
    p[j] = ab;
    p[kHid + j] = aw0;
    p[2 * kHid + j] = aw1;
    if (j < kOut) {
        float s = 0.f;
        for (int r = 0; r < kTileM; ++r) s += d_s[r][j];
        p[3 * kHid + j] = s;
    }
}

// dst[c] = sum_t part[t * ncols + c] for up to four sets of partial sums in one launch: a block
// of kColsumWarps warps per 32 VW columns of one set (lane = VW consecutive columns, so every row
// of partials is read in 32 VW-wide coalesced pieces); warp w adds the rows t in its contiguous
// range with two interleaved accumulators, then the warp sums are added in warp order.  The
// order of every addition is fixed, so the sums are the same on every run.  VW = 4 needs ncols a
// multiple of 4 and 16-byte aligned rows.
constexpr int kColsumWarps = 8;
struct ColsumSet {
    const float *part;
    int64_t nt, ncols;
    float *dst;
    int vw;      // 4 or 1
    int blocks;  // blocks of the launch that serve this set
};
struct ColsumSets {
    ColsumSet s[4];
    int n;
};

template <int VW>
__device__ __forceinline__ void colsum_block(const ColsumSet &g, int64_t blk, float (*ws)[32 * 4 + 1]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nt = g.nt, ncols = g.ncols;
    const float *part = g.part;
    const int64_t c = (blk * 32 + lane) * VW;
    const int64_t t0 = w * nt / kColsumWarps, t1 = (w + 1) * nt / kColsumWarps;
    float a[2][VW] = {};
    if (c < ncols) {
        int64_t t = t0;
        for (; t + 2 <= t1; t += 2) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if constexpr (VW == 4) {
                    const float4 v = __ldg(reinterpret_cast<const float4 *>(part + (t + k) * ncols + c));
                    a[k][0] += v.x;
                    a[k][1] += v.y;
                    a[k][2] += v.z;
                    a[k][3] += v.w;
                } else {
                    a[k][0] += __ldg(part + (t + k) * ncols + c);
                }
            }
        }
        if (t < t1) {
            if constexpr (VW == 4) {
                const float4 v = __ldg(reinterpret_cast<const float4 *>(part + t * ncols + c));
                a[0][0] += v.x;
                a[0][1] += v.y;
                a[0][2] += v.z;
                a[0][3] += v.w;
            } else {
                a[0][0] += __ldg(part + t * ncols + c);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < VW; ++j) ws[w][lane * VW + j] = a[0][j] + a[1][j];
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * VW; i += blockDim.x) {
        const int64_t ci = blk * 32 * VW + i;
        if (ci < ncols) {
            float s = 0.f;
            for (int k = 0; k < kColsumWarps; ++k) s += ws[k][i];
            g.dst[ci] = s;
        }
    }
}

__global__ void __launch_bounds__(kColsumWarps * 32) k_colsum(const ColsumSets S) {
    __shared__ float ws[kColsumWarps][32 * 4 + 1];
    int64_t b = blockIdx.x;
    int k = 0;
    while (k < S.n - 1 && b >= S.s[k].blocks) b -= S.s[k++].blocks;
    if (S.s[k].vw == 4)
        colsum_block<4>(S.s[k], b, ws);
    else
        colsum_block<1>(S.s[k], b, ws);
}

// the column sums of n (<= 4) sets of partials, one launch
int launch_colsums(const ColsumSet *sets, int n, cudaStream_t st) {
    ColsumSets S{};
    S.n = n;
    int64_t total = 0;
    for (int k = 0; k < n; ++k) {
        S.s[k] = sets[k];
        S.s[k].vw = (sets[k].ncols % 4 == 0 && reinterpret_cast<uintptr_t>(sets[k].part) % 16 == 0) ? 4 : 1;
        S.s[k].blocks = (int)((sets[k].ncols + 32 * S.s[k].vw - 1) / (32 * S.s[k].vw));
        total += S.s[k].blocks;
    }
    if (n < 1 || n > 4 || total < 1 || total > 0x7FFFFFFF) return fail(RQ_E_RANGE, "column sums: bad sets");
    k_colsum<<<(unsigned)total, kColsumWarps * 32, 0, st>>>(S);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

__device__ __forceinline__ void write_bf16_copies(const rq_mlp_t &M, int i, float p) {
    if (i >= kOffW1 && i < kOffB1) {
        M.w1b[i - kOffW1] = __bfloat16_as_ushort(__float2bfloat16_rn(p));
    } else if (i >= kOffW2 && i < kOffB2) {
        const int e = i - kOffW2, n = e / kHid, k = e % kHid;
        const unsigned short b = __bfloat16_as_ushort(__float2bfloat16_rn(p));
        M.w2b[e] = b;
        M.w2tb[k * kHid + n] = b;
    }
}

__global__ void k_sync(const rq_mlp_t M) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNParams; i += gridDim.x * blockDim.x)
        write_bf16_copies(M, i, M.params[i]);
}

__global__ void k_adam(const rq_mlp_t M, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNParams; i += gridDim.x * blockDim.x) {
        const float g = M.grads[i];
        const float m = b1 * M.adam_m[i] + (1.f - b1) * g;
        const float v = b2 * M.adam_v[i] + (1.f - b2) * g * g;
        M.adam_m[i] = m;
        M.adam_v[i] = v;
        const float p = M.params[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
        M.params[i] = p;
        write_bf16_copies(M, i, p);
    }
}

template <typename V>
__global__ void k_warm_start(int64_t D, const float *__restrict__ out, V *__restrict__ x0) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < D; k += (int64_t)gridDim.x * blockDim.x) {
        const float a = fminf(out[k * 2], 30.f);
        const double v = (out[k * 2 + 1] < 0.f ? -1.0 : 1.0) * exp((double)a);
        VT<V>::st(x0, k, cx<typename VT<V>::R>{(typename VT<V>::R)v, (typename VT<V>::R)0});
    }
}

// ---------------------------------------------------------------------------------------------
// workspace layout for `rows` rows (Mp = rows rounded up to 128)
// ---------------------------------------------------------------------------------------------
struct MlpLayout {
    int64_t Mp, tiles, nsplit, nsplit1;
    size_t err, z1, h1, h1t, z2, dz2, dz2t, dz1t, colpart1, part2, split2, split1, lossp, total;
};


MlpLayout mlp_layout(int64_t rows) {
    MlpLayout L{};
    L.Mp = (rows + kTileM - 1) / kTileM * kTileM;
    L.tiles = L.Mp / kTileM;
    L.nsplit = std::min<int64_t>(kSplitK, L.Mp / kChunkK);       // dW2: 2 row tiles x nsplit units
    L.nsplit1 = std::min<int64_t>(2 * kSplitK, L.Mp / kChunkK);  // dW1: 1 row tile x nsplit1 units
    size_t off = 0;
    auto take = [&](size_t n) {
        const size_t o = off;
        off += (n + 255) & ~size_t(255);
        return o;
    };
    const size_t act = (size_t)L.Mp * kHid * sizeof(bf16);
    L.err = take(16);
    L.z1 = take(act);
    L.h1 = take(act);
    L.h1t = take(act);
    L.z2 = take(act);
    L.dz2 = take(act);
    L.dz2t = take(act);
    L.dz1t = take(act);
    L.colpart1 = take((size_t)L.tiles * kHid * sizeof(float));  // one row per tile (k_head_bwd) or CTA
    L.part2 = take((size_t)L.tiles * kHeadPart * sizeof(float));
    L.split2 = take((size_t)L.nsplit * kHid * kHid * sizeof(float));
    L.split1 = take((size_t)L.nsplit1 * kHid * kIn * sizeof(float));
    L.lossp = take((size_t)std::max<int64_t>(4096, L.tiles) * sizeof(double));
    L.total = off;
    return L;
}

int check_mlp(const rq_mlp_t *m) {
    if (!m || !m->params || !m->w1b || !m->w2b || !m->w2tb) return fail(RQ_E_ARG, "rq_mlp: null parameter arrays");
    return RQ_OK;
}

int grid_for(int64_t n, int threads = kThreads) {
    int64_t g = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 16;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace
}  // namespace rq

using namespace rq;

RQ_API int rq_mlp_workspace_size(int64_t rows, size_t *bytes) {
    if (rows < 1 || !bytes) return fail(RQ_E_ARG, "rq_mlp_workspace_size: bad arguments");
    *bytes = mlp_layout(rows).total;
    return RQ_OK;
}

RQ_API int rq_mlp_sync(const rq_mlp_t *m, void *stream) {
    RQ_TRY(check_mlp(m));
    k_sync<<<grid_for(kNParams), kThreads, 0, as_stream(stream)>>>(*m);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_mlp_features(const uint64_t *states, int64_t D, double U, uint16_t *x, void *stream) {
    if (!states || !x || D < 1) return fail(RQ_E_ARG, "rq_mlp_features: bad arguments");
    k_features<<<grid_for(D), kThreads, 0, as_stream(stream)>>>(states, D, U, reinterpret_cast<bf16 *>(x));
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_mlp_sample(const uint64_t *states, int64_t D, const double *U, const float *psi, int32_t P,
                         uint64_t seed, int64_t step, int64_t rows, uint16_t *x, uint16_t *xt, float *tgt,
                         void *stream) {
    if (!states || !U || !psi || !x || !xt || !tgt || D < 1 || P < 1 || rows < 1)
        return fail(RQ_E_ARG, "rq_mlp_sample: bad arguments");
    k_sample<<<grid_for(rows), kThreads, 0, as_stream(stream)>>>(states, D, U, psi, P, seed, step, rows,
                                                                 reinterpret_cast<bf16 *>(x),
                                                                 reinterpret_cast<bf16 *>(xt), tgt);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

namespace rq {
namespace {

// layer 1: Z1 = X W1^T + b1 and H1 = GELU(Z1), row-major, and H1 feature-major (the B operand of dW2)
int layer1(const rq_mlp_t *m, int64_t rows, const uint16_t *x, const MlpLayout &L, char *w, int *err,
           cudaStream_t st) {
    GemmArgs g{};
    g.M = rows;
    g.nsplit = 1;
    g.bias = m->params + kOffB1;
    g.z_rm = reinterpret_cast<bf16 *>(w + L.z1);
    g.h_rm = reinterpret_cast<bf16 *>(w + L.h1);
    g.h_fm = reinterpret_cast<bf16 *>(w + L.h1t);
    g.ld_fm = L.Mp;
    g.err = err;
    return launch_gemm<kHid, EPI_HIDDEN>(reinterpret_cast<const bf16 *>(x), kIn,
                                         reinterpret_cast<const bf16 *>(m->w1b), kIn, kIn, g, st);
}

// dZ1 = (dZ2 W2) * GELU'(Z1) feature-major with the b1 partial sums, dW2 = dZ2^T H1 and
// dW1 = dZ1^T X split over the rows (column-major partial products), and the sums of every set of
// partials into m->grads
int backward_tail(const rq_mlp_t *m, int64_t rows, const uint16_t *xt, const MlpLayout &L, char *w, int *err,
                  const float *part2, int64_t part2_rows, cudaStream_t st) {
    GemmArgs g{};
    g.M = rows;
    g.nsplit = 1;
    g.zin_rm = reinterpret_cast<const bf16 *>(w + L.z1);
    g.h_fm = reinterpret_cast<bf16 *>(w + L.dz1t);
    g.ld_fm = L.Mp;
    g.colpart = reinterpret_cast<float *>(w + L.colpart1);
    g.err = err;
    int64_t grid1 = 0;
    RQ_TRY((launch_gemm<kHid, EPI_DGELU>(reinterpret_cast<const bf16 *>(w + L.dz2), kHid,
                                         reinterpret_cast<const bf16 *>(m->w2tb), kHid, kHid, g, st, &grid1)));
    // dW2^T = H1^T dZ2: A = H1 feature-major (rows n), B = dZ2 feature-major (columns j); the
    // column-major partial product [j][n] is dW2 in its row-major layout
    GemmArgs a{};
    a.M = kHid;
    a.nsplit = L.nsplit;
    a.out = reinterpret_cast<float *>(w + L.split2);
    a.split_cm = 1;
    a.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_F32>(reinterpret_cast<const bf16 *>(w + L.h1t), L.Mp,
                                       reinterpret_cast<const bf16 *>(w + L.dz2t), L.Mp, L.Mp, a, st)));
    // dW1^T = X^T dZ1: a 64-row A tile (rows 64..127 read as zeros), one row tile, twice the splits
    GemmArgs b{};
    b.M = kIn;
    b.nsplit = L.nsplit1;
    b.out = reinterpret_cast<float *>(w + L.split1);
    b.split_cm = 1;
    b.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_F32>(reinterpret_cast<const bf16 *>(xt), L.Mp,
                                       reinterpret_cast<const bf16 *>(w + L.dz1t), L.Mp, L.Mp, b, st)));
    const ColsumSet sets[4] = {
        {reinterpret_cast<const float *>(w + L.split1), L.nsplit1, kHid * kIn, m->grads + kOffW1, 0, 0},
        {reinterpret_cast<const float *>(w + L.colpart1), grid1, kHid, m->grads + kOffB1, 0, 0},
        {reinterpret_cast<const float *>(w + L.split2), L.nsplit, kHid * kHid, m->grads + kOffW2, 0, 0},
        {part2, part2_rows, kHeadPart, m->grads + kOffB2, 0, 0}};
    return launch_colsums(sets, 4, st);
}

}  // namespace
}  // namespace rq

RQ_API int rq_mlp_fwd(const rq_mlp_t *m, int64_t rows, const uint16_t *x, float *out, void *ws, void *stream) {
    RQ_TRY(check_mlp(m));
    if (rows < 1 || !x || !out || !ws) return fail(RQ_E_ARG, "rq_mlp_fwd: bad arguments");
    const MlpLayout L = mlp_layout(rows);
    char *w = static_cast<char *>(ws);
    cudaStream_t st = as_stream(stream);
    int *err = reinterpret_cast<int *>(w + L.err);
    RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    RQ_TRY(layer1(m, rows, x, L, w, err, st));
    GemmArgs h{};
    h.M = rows;
    h.nsplit = 1;
    h.bias = m->params + kOffB2;
    h.z_rm = reinterpret_cast<bf16 *>(w + L.z2);
    h.out = out;
    h.w3 = m->params + kOffW3;
    h.b3 = m->params + kOffB3;
    h.err = err;
    return launch_gemm<kHid, EPI_HEAD>(reinterpret_cast<const bf16 *>(w + L.h1), kHid,
                                       reinterpret_cast<const bf16 *>(m->w2b), kHid, kHid, h, st);
}

RQ_API int rq_mlp_infer(const rq_mlp_t *m, int64_t rows, const uint16_t *x, float *out, void *ws, void *stream) {
    RQ_TRY(check_mlp(m));
    if (rows < 1 || !x || !out || !ws) return fail(RQ_E_ARG, "rq_mlp_infer: bad arguments");
    const MlpLayout L = mlp_layout(rows);
    char *w = static_cast<char *>(ws);
    cudaStream_t st = as_stream(stream);
    int *err = reinterpret_cast<int *>(w + L.err);
    RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    GemmArgs g{};
    g.M = rows;
    g.nsplit = 1;
    g.bias = m->params + kOffB1;
    g.h_rm = reinterpret_cast<bf16 *>(w + L.h1);
    g.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_HIDDEN>(reinterpret_cast<const bf16 *>(x), kIn,
                                          reinterpret_cast<const bf16 *>(m->w1b), kIn, kIn, g, st)));
    GemmArgs h{};
    h.M = rows;
    h.nsplit = 1;
    h.bias = m->params + kOffB2;
    h.out = out;
    h.w3 = m->params + kOffW3;
    h.b3 = m->params + kOffB3;
    h.err = err;
    return launch_gemm<kHid, EPI_HEAD>(reinterpret_cast<const bf16 *>(w + L.h1), kHid,
                                       reinterpret_cast<const bf16 *>(m->w2b), kHid, kHid, h, st);
}

RQ_API int rq_mlp_loss(int64_t rows, const float *out, const float *tgt, float *dout, double *loss, void *ws,
                       void *stream) {
    if (rows < 1 || !out || !tgt || !dout || !ws) return fail(RQ_E_ARG, "rq_mlp_loss: bad arguments");
    const MlpLayout L = mlp_layout(rows);
    double *part = reinterpret_cast<double *>(static_cast<char *>(ws) + L.lossp);
    const int grid = std::min(grid_for(rows), 4096);
    cudaStream_t st = as_stream(stream);
    k_loss<<<grid, kThreads, 0, st>>>(rows, out, tgt, dout, part);
    if (loss) k_loss_sum<<<1, kThreads, 0, st>>>(part, grid, rows, loss);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_mlp_bwd(const rq_mlp_t *m, int64_t rows, const uint16_t *xt, const float *dout, void *ws,
                      void *stream) {
    RQ_TRY(check_mlp(m));
    if (!m->grads || !xt || !dout || !ws) return fail(RQ_E_ARG, "rq_mlp_bwd: null argument");
    if (rows < kTileM || rows % kTileM != 0) return fail(RQ_E_ARG, "rq_mlp_bwd: rows must be a multiple of 128");
    const MlpLayout L = mlp_layout(rows);
    char *w = static_cast<char *>(ws);
    cudaStream_t st = as_stream(stream);
    int *err = reinterpret_cast<int *>(w + L.err);
    float *part2 = reinterpret_cast<float *>(w + L.part2);
    k_head_bwd<<<(unsigned)L.tiles, kHid, 0, st>>>(reinterpret_cast<const bf16 *>(w + L.z2), dout, m->params,
                                                   L.Mp, reinterpret_cast<bf16 *>(w + L.dz2),
                                                   reinterpret_cast<bf16 *>(w + L.dz2t), part2);
    RQ_CUDA(cudaGetLastError());
    return backward_tail(m, rows, xt, L, w, err, part2, L.tiles, st);
}

RQ_API int rq_mlp_train(const rq_mlp_t *m, int64_t rows, const uint16_t *x, const uint16_t *xt, const float *tgt,
                        float *out, double *loss, void *ws, void *stream) {
    RQ_TRY(check_mlp(m));
    if (!m->grads || !x || !xt || !tgt || !ws) return fail(RQ_E_ARG, "rq_mlp_train: null argument");
    if (rows < kTileM || rows % kTileM != 0) return fail(RQ_E_ARG, "rq_mlp_train: rows must be a multiple of 128");
    const MlpLayout L = mlp_layout(rows);
    char *w = static_cast<char *>(ws);
    cudaStream_t st = as_stream(stream);
    int *err = reinterpret_cast<int *>(w + L.err);
    RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    RQ_TRY(layer1(m, rows, x, L, w, err, st));
    // layer 2 with the output layer, the loss and its gradient back to dZ2 in one epilogue
    GemmArgs h{};
    h.M = rows;
    h.nsplit = 1;
    h.bias = m->params + kOffB2;
    h.out = out;
    h.w3 = m->params + kOffW3;
    h.b3 = m->params + kOffB3;
    h.tgt = tgt;
    h.inv_rows = 1.f / (float)rows;
    h.dz_rm = reinterpret_cast<bf16 *>(w + L.dz2);
    h.h_fm = reinterpret_cast<bf16 *>(w + L.dz2t);
    h.ld_fm = L.Mp;
    h.colpart = reinterpret_cast<float *>(w + L.part2);
    h.losspart = reinterpret_cast<double *>(w + L.lossp);
    h.err = err;
    int64_t grid2 = 0;
    RQ_TRY((launch_gemm<kHid, EPI_HEAD_TRAIN>(reinterpret_cast<const bf16 *>(w + L.h1), kHid,
                                              reinterpret_cast<const bf16 *>(m->w2b), kHid, kHid, h, st, &grid2)));
    if (loss) {
        k_loss_sum<<<1, kThreads, 0, st>>>(reinterpret_cast<const double *>(w + L.lossp), (int)grid2, rows, loss);
        RQ_CUDA(cudaGetLastError());
    }
    return backward_tail(m, rows, xt, L, w, err, reinterpret_cast<const float *>(w + L.part2), grid2, st);
}

RQ_API int rq_mlp_step(const rq_mlp_t *m, int32_t t, float lr, float beta1, float beta2, float eps,
                       void *stream) {
    RQ_TRY(check_mlp(m));
    if (!m->grads || !m->adam_m || !m->adam_v || t < 1) return fail(RQ_E_ARG, "rq_mlp_step: bad arguments");
    const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
    k_adam<<<grid_for(kNParams), kThreads, 0, as_stream(stream)>>>(*m, lr, beta1, beta2, eps, c1, c2);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_mlp_warm_start(int64_t D, const float *out, int32_t vtype, void *x0, void *stream) {
    if (D < 1 || !out || !x0) return fail(RQ_E_ARG, "rq_mlp_warm_start: bad arguments");
    cudaStream_t st = as_stream(stream);
    const int grid = grid_for(D);
    switch (vtype) {
        case RQ_F32: k_warm_start<float><<<grid, kThreads, 0, st>>>(D, out, static_cast<float *>(x0)); break;
        case RQ_F64: k_warm_start<double><<<grid, kThreads, 0, st>>>(D, out, static_cast<double *>(x0)); break;
        case RQ_C64: k_warm_start<float2><<<grid, kThreads, 0, st>>>(D, out, static_cast<float2 *>(x0)); break;
        case RQ_C128: k_warm_start<double2><<<grid, kThreads, 0, st>>>(D, out, static_cast<double2 *>(x0)); break;
        default: return fail(RQ_E_ARG, "rq_mlp_warm_start: bad vtype");
    }
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

RQ_API int rq_bf16_gemm(const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb, int64_t M, int32_t N,
                        int64_t K, float *C, void *ws, void *stream) {
    if (!A || !B || !C || !ws || M < 1 || K < kChunkK || K % kChunkK != 0 || lda % 8 != 0 || ldb % 8 != 0 ||
        lda < K || ldb < K)
        return fail(RQ_E_ARG, "rq_bf16_gemm: bad arguments");
    if (N != 64 && N != 256) return fail(RQ_E_ARG, "rq_bf16_gemm: N must be 64 or 256");
    cudaStream_t st = as_stream(stream);
    int *err = static_cast<int *>(ws);
    RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    GemmArgs g{};
    g.M = M;
    g.nsplit = 1;
    g.out = C;
    g.err = err;
    const bf16 *a = reinterpret_cast<const bf16 *>(A), *b = reinterpret_cast<const bf16 *>(B);
    if (N == 64) return launch_gemm<64, EPI_F32>(a, lda, b, ldb, K, g, st);
    return launch_gemm<256, EPI_F32>(a, lda, b, ldb, K, g, st);
}
