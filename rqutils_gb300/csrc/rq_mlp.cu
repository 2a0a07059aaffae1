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
#include <cuda_bf16.h>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kIn = RQ_MLP_IN, kHid = RQ_MLP_HIDDEN, kOut = RQ_MLP_OUT;
constexpr int kTileM = 128, kChunkK = 64, kGemmThreads = 128;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kHid * kIn, kOffW2 = kOffB1 + kHid,
              kOffB2 = kOffW2 + kHid * kHid, kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kOut * kHid,
              kNParams = kOffB3 + kOut;
static_assert(kNParams == RQ_MLP_NPARAMS, "parameter layout");
constexpr int kHeadPart = kHid + kOut * kHid + kOut;  // db2 | dW3 | db3 partial sums per tile
constexpr long long kWaitCycles = 2000000000LL;

enum Epi { EPI_F32 = 0, EPI_HIDDEN = 1, EPI_HEAD = 2, EPI_DGELU = 3 };

// ---------------------------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
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
// bounded wait for the phase of the given parity; false when the limit expired
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
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

// shared-memory matrix descriptor: no swizzle, K-major canonical layout
__device__ __forceinline__ uint64_t make_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;
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

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"  // in the same statement: the outputs exist after the wait
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// ---------------------------------------------------------------------------------------------
// activations
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float dgelu(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---------------------------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------------------------
struct GemmArgs {
    const bf16 *A;
    int64_t lda;
    int64_t M;  // rows of A; rows >= M are zero-filled and not stored
    const bf16 *B;
    int64_t ldb;
    int64_t kper;  // K per blockIdx.y, a multiple of 64
    const float *bias;
    bf16 *z_rm;     // pre-activations, row-major [M][N] (HIDDEN, HEAD; optional)
    bf16 *h_rm;     // activations, row-major [M][N] (HIDDEN)
    bf16 *h_fm;     // feature-major [N][ld_fm] (HIDDEN: activations, optional; DGELU: gradients)
    int64_t ld_fm;
    const bf16 *zin_rm;  // pre-activations read by DGELU, row-major [M][N]
    float *out;          // F32: [gridDim.y][M][N]; HEAD: [M][2]
    const float *w3;     // HEAD: [2][N]
    const float *b3;     // HEAD: [2]
    float *colpart;      // DGELU: [gridDim.x][N] column sums of the gradient
    int *err;
};

__device__ __forceinline__ uint32_t cm_offset(int r, int kc) {
    return (uint32_t)((r >> 3) * 1024 + kc * 128 + (r & 7) * 16);
}

// rows [row0, row0 + R) x K [k0, k0 + 64) of P into the core-matrix layout at sbase
template <int R>
__device__ __forceinline__ void load_chunk(uint32_t sbase, const bf16 *P, int64_t ld, int64_t row0,
                                           int64_t nrows, int64_t k0) {
    for (int i = threadIdx.x; i < R * 8; i += kGemmThreads) {
        const int r = i >> 3, c = i & 7;
        const int64_t gr = row0 + r;
        const bool ok = gr < nrows;
        const bf16 *src = P + (ok ? gr : row0 < nrows ? row0 : 0) * ld + k0 + c * 8;
        cp_async16(sbase + cm_offset(r, c), src, ok ? 16 : 0);
    }
}

template <int N>
constexpr uint32_t gemm_smem_bytes() {
    return 2u * (uint32_t)(kTileM * kChunkK * 2 + N * kChunkK * 2);
}

template <int N, int EPI>
__global__ void __launch_bounds__(kGemmThreads, 1) k_gemm(const GemmArgs g) {
    static_assert(N == 64 || N == 256, "N is 64 or 256");
    extern __shared__ __align__(1024) unsigned char smem[];
    constexpr uint32_t kA = kTileM * kChunkK * 2;
    constexpr uint32_t kStage = kA + N * kChunkK * 2;
    constexpr uint32_t kIdesc = make_idesc(kTileM, N);
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_s;
    __shared__ int abort_s;
    __shared__ float colsum_s[4][EPI == EPI_DGELU ? N : 1];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kTileM;
    const int64_t kb = (int64_t)blockIdx.y * g.kper;
    const int nchunks = (int)(g.kper / kChunkK);
    if (warp == 0) tmem_alloc(&tmem_s, (uint32_t)N);
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        fence_mbar_init();
        abort_s = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_s;
    const uint32_t sbase = smem_u32(smem);

    for (int c = 0; c < nchunks; ++c) {
        const int s = c & 1;
        if (c >= 2 && tid == 0 && !mbar_wait(&mbar[s], (uint32_t)(((c - 2) >> 1) & 1))) abort_s = 1;
        __syncthreads();
        if (abort_s) break;
        const uint32_t sa = sbase + (uint32_t)s * kStage, sb = sa + kA;
        const int64_t k0 = kb + (int64_t)c * kChunkK;
        load_chunk<kTileM>(sa, g.A, g.lda, m0, g.M, k0);
        load_chunk<N>(sb, g.B, g.ldb, 0, N, k0);
        cp_async_commit();
        cp_async_wait_all();
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < kChunkK / 16; ++kk) {
                const uint64_t ad = make_sdesc(sa + (uint32_t)kk * 256u, 128u, 1024u);
                const uint64_t bd = make_sdesc(sb + (uint32_t)kk * 256u, 128u, 1024u);
                mma_bf16(tmem, ad, bd, kIdesc, (c > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(&mbar[s]);
        }
    }
    // the last commit covers every MMA issued before it
    if (tid == 0 && !abort_s && nchunks > 0) {
        const int c = nchunks - 1;
        if (!mbar_wait(&mbar[c & 1], (uint32_t)((c >> 1) & 1))) abort_s = 1;
    }
    __syncthreads();
    tc_fence_after();
    const bool aborted = abort_s != 0;
    if (aborted && tid == 0 && g.err) atomicExch(g.err, RQ_E_CUDA);

    if (!aborted) {
        const int64_t m = m0 + tid;
        const bool valid = m < g.M;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        float o0 = 0.f, o1 = 0.f;
#pragma unroll 1
        for (int j0 = 0; j0 < N; j0 += 16) {
            float v[16];
            tmem_ld16(taddr + (uint32_t)j0, v);
            if constexpr (EPI == EPI_F32) {
                if (valid) {
                    float4 *dst = reinterpret_cast<float4 *>(g.out + ((int64_t)blockIdx.y * g.M + m) * N + j0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
            } else if constexpr (EPI == EPI_HIDDEN || EPI == EPI_HEAD) {
                __align__(16) bf16 zb[16], hb[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const float z = v[q] + __ldg(g.bias + j0 + q);
                    const float h = gelu(z);
                    zb[q] = __float2bfloat16_rn(z);
                    hb[q] = __float2bfloat16_rn(h);
                    if constexpr (EPI == EPI_HEAD) {
                        o0 += h * __ldg(g.w3 + j0 + q);
                        o1 += h * __ldg(g.w3 + N + j0 + q);
                    }
                }
                if (valid) {
                    if (g.z_rm) {
                        uint4 *dz = reinterpret_cast<uint4 *>(g.z_rm + m * N + j0);
                        dz[0] = reinterpret_cast<const uint4 *>(zb)[0];
                        dz[1] = reinterpret_cast<const uint4 *>(zb)[1];
                    }
                    if constexpr (EPI == EPI_HIDDEN) {
                        uint4 *dh = reinterpret_cast<uint4 *>(g.h_rm + m * N + j0);
                        dh[0] = reinterpret_cast<const uint4 *>(hb)[0];
                        dh[1] = reinterpret_cast<const uint4 *>(hb)[1];
                        if (g.h_fm) {
#pragma unroll
                            for (int q = 0; q < 16; ++q) g.h_fm[(int64_t)(j0 + q) * g.ld_fm + m] = hb[q];
                        }
                    }
                }
            } else {  // EPI_DGELU
                __align__(16) bf16 zin[16];
                if (valid) {
                    const uint4 *src = reinterpret_cast<const uint4 *>(g.zin_rm + m * N + j0);
                    reinterpret_cast<uint4 *>(zin)[0] = src[0];
                    reinterpret_cast<uint4 *>(zin)[1] = src[1];
                }
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const float dz = valid ? v[q] * dgelu(__bfloat162float(zin[q])) : 0.f;
                    if (valid) g.h_fm[(int64_t)(j0 + q) * g.ld_fm + m] = __float2bfloat16_rn(dz);
                    float sum = dz;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                    if (lane == 0) colsum_s[warp][j0 + q] = sum;
                }
            }
        }
        if (EPI == EPI_HEAD && valid) {
            g.out[m * 2] = o0 + __ldg(g.b3);
            g.out[m * 2 + 1] = o1 + __ldg(g.b3 + 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    if constexpr (EPI == EPI_DGELU) {
        if (!aborted)
            for (int j = tid; j < N; j += kGemmThreads)
                g.colpart[(int64_t)blockIdx.x * N + j] = colsum_s[0][j] + colsum_s[1][j] + colsum_s[2][j] + colsum_s[3][j];
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, (uint32_t)N);
    }
}

template <int N, int EPI>
int launch_gemm(const GemmArgs &g, int64_t tiles, int64_t splits, cudaStream_t st) {
    constexpr uint32_t smem = gemm_smem_bytes<N>();
    thread_local KernelLaunchCache table[kMaxCachedDevices];
    KernelLaunchCache *c = nullptr;
    int per_sm = 1;
    RQ_TRY(cache_slot(table, &c));
    RQ_TRY(configure_kernel(k_gemm<N, EPI>, *c, smem, kGemmThreads, &per_sm));
    if (tiles < 1 || splits < 1 || tiles > 0x7FFFFFFF || splits > 65535)
        return fail(RQ_E_RANGE, "bf16 GEMM: grid out of range");
    k_gemm<N, EPI><<<dim3((unsigned)tiles, (unsigned)splits), kGemmThreads, smem, st>>>(g);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
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

__global__ void k_loss_sum(const double *__restrict__ part, int n, int64_t rows, double *loss) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.;
        for (int i = 0; i < n; ++i) s += part[i];
        *loss = s / (double)rows;
    }
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

// dst[c] = sum_t part[t * ncols + c]: a block of kColsumWarps warps per 32 columns (lane =
// column: every row of partials is read coalesced); warp w adds the rows t in its contiguous
// range with four interleaved accumulators, then warp 0 adds the warp sums in warp order.  The
// order of every addition is fixed, so the sums are the same on every run.
constexpr int kColsumWarps = 32;
__global__ void __launch_bounds__(kColsumWarps * 32)
k_colsum(const float *__restrict__ part, int64_t nt, int64_t ncols, float *__restrict__ dst) {
    __shared__ float ws[kColsumWarps][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t c = (int64_t)blockIdx.x * 32 + lane;
    const int64_t t0 = w * nt / kColsumWarps, t1 = (w + 1) * nt / kColsumWarps;
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    if (c < ncols) {
        int64_t t = t0;
        for (; t + 4 <= t1; t += 4) {
#pragma unroll
            for (int k = 0; k < 4; ++k) a[k] += __ldg(part + (t + k) * ncols + c);
        }
        for (int k = 0; t < t1; ++t, ++k) a[k] += __ldg(part + t * ncols + c);
    }
    ws[w][lane] = (a[0] + a[1]) + (a[2] + a[3]);
    __syncthreads();
    if (w == 0 && c < ncols) {
        float s = 0.f;
        for (int k = 0; k < kColsumWarps; ++k) s += ws[k][lane];
        dst[c] = s;
    }
}

int launch_colsum(const float *part, int64_t nt, int64_t ncols, float *dst, cudaStream_t st) {
    k_colsum<<<(unsigned)((ncols + 31) / 32), kColsumWarps * 32, 0, st>>>(part, nt, ncols, dst);
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
    int64_t Mp, tiles, nsplit;
    size_t err, z1, h1, h1t, z2, dz2, dz2t, dz1t, colpart1, part2, split2, split1, lossp, total;
};

int64_t pick_splits(int64_t Mp) {
    int64_t s = 64;
    while (s > 1 && Mp % (s * kChunkK) != 0) s >>= 1;
    return s;
}

MlpLayout mlp_layout(int64_t rows) {
    MlpLayout L{};
    L.Mp = (rows + kTileM - 1) / kTileM * kTileM;
    L.tiles = L.Mp / kTileM;
    L.nsplit = pick_splits(L.Mp);
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
    L.colpart1 = take((size_t)L.tiles * kHid * sizeof(float));
    L.part2 = take((size_t)L.tiles * kHeadPart * sizeof(float));
    L.split2 = take((size_t)L.nsplit * kHid * kHid * sizeof(float));
    L.split1 = take((size_t)L.nsplit * kHid * kIn * sizeof(float));
    L.lossp = take(4096 * sizeof(double));
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

RQ_API int rq_mlp_fwd(const rq_mlp_t *m, int64_t rows, const uint16_t *x, float *out, void *ws, void *stream) {
    RQ_TRY(check_mlp(m));
    if (rows < 1 || !x || !out || !ws) return fail(RQ_E_ARG, "rq_mlp_fwd: bad arguments");
    const MlpLayout L = mlp_layout(rows);
    char *w = static_cast<char *>(ws);
    cudaStream_t st = as_stream(stream);
    int *err = reinterpret_cast<int *>(w + L.err);
    RQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    GemmArgs g{};
    g.A = reinterpret_cast<const bf16 *>(x);
    g.lda = kIn;
    g.M = rows;
    g.B = reinterpret_cast<const bf16 *>(m->w1b);
    g.ldb = kIn;
    g.kper = kIn;
    g.bias = m->params + kOffB1;
    g.z_rm = reinterpret_cast<bf16 *>(w + L.z1);
    g.h_rm = reinterpret_cast<bf16 *>(w + L.h1);
    g.h_fm = reinterpret_cast<bf16 *>(w + L.h1t);
    g.ld_fm = L.Mp;
    g.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_HIDDEN>(g, L.tiles, 1, st)));
    GemmArgs h{};
    h.A = reinterpret_cast<const bf16 *>(w + L.h1);
    h.lda = kHid;
    h.M = rows;
    h.B = reinterpret_cast<const bf16 *>(m->w2b);
    h.ldb = kHid;
    h.kper = kHid;
    h.bias = m->params + kOffB2;
    h.z_rm = reinterpret_cast<bf16 *>(w + L.z2);
    h.out = out;
    h.w3 = m->params + kOffW3;
    h.b3 = m->params + kOffB3;
    h.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_HEAD>(h, L.tiles, 1, st)));
    return RQ_OK;
}

RQ_API int rq_mlp_loss(int64_t rows, const float *out, const float *tgt, float *dout, double *loss, void *ws,
                       void *stream) {
    if (rows < 1 || !out || !tgt || !dout || !ws) return fail(RQ_E_ARG, "rq_mlp_loss: bad arguments");
    const MlpLayout L = mlp_layout(rows);
    double *part = reinterpret_cast<double *>(static_cast<char *>(ws) + L.lossp);
    const int grid = std::min(grid_for(rows), 4096);
    cudaStream_t st = as_stream(stream);
    k_loss<<<grid, kThreads, 0, st>>>(rows, out, tgt, dout, part);
    if (loss) k_loss_sum<<<1, 32, 0, st>>>(part, grid, rows, loss);
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
    bf16 *dz2 = reinterpret_cast<bf16 *>(w + L.dz2), *dz2t = reinterpret_cast<bf16 *>(w + L.dz2t);
    float *part2 = reinterpret_cast<float *>(w + L.part2);
    k_head_bwd<<<(unsigned)L.tiles, kHid, 0, st>>>(reinterpret_cast<const bf16 *>(w + L.z2), dout, m->params,
                                                   L.Mp, dz2, dz2t, part2);
    RQ_CUDA(cudaGetLastError());
    // dZ1 = (dZ2 W2) * GELU'(Z1), written feature-major, with the b1 column sums
    GemmArgs g{};
    g.A = dz2;
    g.lda = kHid;
    g.M = rows;
    g.B = reinterpret_cast<const bf16 *>(m->w2tb);
    g.ldb = kHid;
    g.kper = kHid;
    g.zin_rm = reinterpret_cast<const bf16 *>(w + L.z1);
    g.h_fm = reinterpret_cast<bf16 *>(w + L.dz1t);
    g.ld_fm = L.Mp;
    g.colpart = reinterpret_cast<float *>(w + L.colpart1);
    g.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_DGELU>(g, L.tiles, 1, st)));
    // dW2 = dZ2^T H1 and dW1 = dZ1^T X, split over the rows (K) and summed in split order
    GemmArgs a{};
    a.A = dz2t;
    a.lda = L.Mp;
    a.M = kHid;
    a.B = reinterpret_cast<const bf16 *>(w + L.h1t);
    a.ldb = L.Mp;
    a.kper = L.Mp / L.nsplit;
    a.out = reinterpret_cast<float *>(w + L.split2);
    a.err = err;
    RQ_TRY((launch_gemm<kHid, EPI_F32>(a, kHid / kTileM, L.nsplit, st)));
    GemmArgs b{};
    b.A = reinterpret_cast<const bf16 *>(w + L.dz1t);
    b.lda = L.Mp;
    b.M = kHid;
    b.B = reinterpret_cast<const bf16 *>(xt);
    b.ldb = L.Mp;
    b.kper = L.Mp / L.nsplit;
    b.out = reinterpret_cast<float *>(w + L.split1);
    b.err = err;
    RQ_TRY((launch_gemm<kIn, EPI_F32>(b, kHid / kTileM, L.nsplit, st)));
    RQ_TRY(launch_colsum(reinterpret_cast<const float *>(w + L.split1), L.nsplit, kHid * kIn,
                         m->grads + kOffW1, st));
    RQ_TRY(launch_colsum(reinterpret_cast<const float *>(w + L.colpart1), L.tiles, kHid,
                         m->grads + kOffB1, st));
    RQ_TRY(launch_colsum(reinterpret_cast<const float *>(w + L.split2), L.nsplit, kHid * kHid,
                         m->grads + kOffW2, st));
    RQ_TRY(launch_colsum(part2, L.tiles, kHeadPart, m->grads + kOffB2, st));
    return RQ_OK;
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
    g.A = reinterpret_cast<const bf16 *>(A);
    g.lda = lda;
    g.M = M;
    g.B = reinterpret_cast<const bf16 *>(B);
    g.ldb = ldb;
    g.kper = K;
    g.out = C;
    g.err = err;
    const int64_t tiles = (M + kTileM - 1) / kTileM;
    if (N == 64) return launch_gemm<64, EPI_F32>(g, tiles, 1, st);
    return launch_gemm<256, EPI_F32>(g, tiles, 1, st);
}
