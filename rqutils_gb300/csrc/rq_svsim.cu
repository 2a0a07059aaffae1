// State-vector simulation of Pauli-rotation circuits (the reference's svsim, svsim.py:88-122).
//
// A gate is (x, z, c, s): out[i] = i s (-1)^popcount(i & z) state[i ^ x] + c state[i] (the c term
// is dropped when c == 0, as the reference does).  Runs of consecutive diagonal gates (x = 0) are
// applied in one pass, each amplitude going through the gates of the run in order in registers.
// A non-diagonal gate is one in-place pass over the pairs (i, i ^ x): each thread reads both
// amplitudes of its pair and writes both outputs.  Products and sums are rounded one at a time
// (no fused multiply-add) in the order of the reference's complex arithmetic, so results equal
// the reference arithmetic bit for bit (up to the sign of zero results).
#include <vector>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {
namespace {

struct Gate {
    uint64_t x, z;
    double c, s;
};

// out = i s sigma v_src + c v_self   (sigma = +-1).  (0 + i a)(re + i im) = (0 re - a im) +
// i (0 im + a re); the 0 x terms only decide the sign of a zero result and are left out
// (GB300 issues FP64 at a small fraction of its FP32 rate), as is the product s sigma (exact).
__device__ __forceinline__ double2 rot(double c, double s, bool neg, double2 self, double2 src, bool with_c) {
    const double a = neg ? -s : s;
    double re = -__dmul_rn(a, src.y);
    double im = __dmul_rn(a, src.x);
    if (with_c) {
        re = __dadd_rn(re, __dmul_rn(c, self.x));
        im = __dadd_rn(im, __dmul_rn(c, self.y));
    }
    return make_double2(re, im);
}

__device__ __forceinline__ bool parity_odd(uint64_t i, uint64_t z) { return __popcll(i & z) & 1; }

// gates [g0, g1) are diagonal
__global__ void k_diag_run(double2 *__restrict__ psi, uint64_t N, const Gate *__restrict__ gates, int g0, int g1) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        double2 v = psi[i];
        for (int g = g0; g < g1; ++g) {
            const Gate G = gates[g];
            v = rot(G.c, G.s, parity_odd(i, G.z), v, v, G.c != 0.0);
        }
        psi[i] = v;
    }
}

// one non-diagonal gate, in place over pairs (i, i ^ x); lb = lowest set bit of x
__global__ void k_pair(double2 *__restrict__ psi, uint64_t N, const Gate *__restrict__ gates, int g, int lb) {
    const Gate G = gates[g];
    const uint64_t half = N >> 1;
    const uint64_t low = (1ULL << lb) - 1ULL;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < half; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = ((t & ~low) << 1) | (t & low);  // bit lb of i is 0
        const uint64_t j = i ^ G.x;
        const double2 a = psi[i], b = psi[j];
        const bool wc = G.c != 0.0;
        psi[i] = rot(G.c, G.s, parity_odd(i, G.z), a, b, wc);
        psi[j] = rot(G.c, G.s, parity_odd(j, G.z), b, a, wc);
    }
}

int grid_for(uint64_t n) {
    uint64_t g = (n + kThreads - 1) / kThreads;
    const uint64_t cap = (uint64_t)sm_count() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace
}  // namespace rq

using namespace rq;

RQ_API int rq_svsim(const uint64_t *x, const uint64_t *z, const double *cosv, const double *sinv, int32_t ngates,
                    int32_t n, void *state, void *gates_scratch, void *stream) {
    if (!x || !z || !cosv || !sinv || !state || ngates < 0 || n < 1 || n > 40 || (ngates > 0 && !gates_scratch))
        return fail(RQ_E_ARG, "rq_svsim: bad arguments (1 <= n <= 40)");
    const uint64_t N = 1ULL << n;
    std::vector<Gate> h(ngates);
    for (int g = 0; g < ngates; ++g) {
        if ((x[g] >> n) != 0 || (z[g] >> n) != 0) return fail(RQ_E_ARG, "rq_svsim: a gate acts beyond n qubits");
        h[g] = Gate{x[g], z[g], cosv[g], sinv[g]};
    }
    if (ngates == 0) return RQ_OK;
    cudaStream_t st = as_stream(stream);
    Gate *dg = static_cast<Gate *>(gates_scratch);
    RQ_CUDA(cudaMemcpyAsync(dg, h.data(), sizeof(Gate) * ngates, cudaMemcpyHostToDevice, st));
    double2 *psi = static_cast<double2 *>(state);
    int g = 0;
    while (g < ngates) {
        if (h[g].x == 0) {
            int e = g;
            while (e < ngates && h[e].x == 0) ++e;
            k_diag_run<<<grid_for(N), kThreads, 0, st>>>(psi, N, dg, g, e);
            g = e;
        } else {
            const int lb = __builtin_ctzll(h[g].x);
            k_pair<<<grid_for(N >> 1), kThreads, 0, st>>>(psi, N, dg, g, lb);
            ++g;
        }
    }
    RQ_CUDA(cudaGetLastError());
    RQ_CUDA(cudaStreamSynchronize(st));  // the host gate list is freed on return
    return RQ_OK;
}
