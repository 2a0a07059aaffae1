// Pauli-sum consolidation and grouping on the device: the array work of
// PauliSumXZ.from_paulisum (rqutils/paulis/symplectic.py:58-125) for terms already parsed into
// X / Z masks (bit q = qubit q).
//
//   1. drop exact-zero coefficients (symplectic.py:68-69);
//   2. merge equal strings (symplectic.py:70-73: np.unique of the labels, the coefficients of a
//      label summed): a stable radix sort of the term indices by the string's lexicographic key
//      (character 0 = qubit n-1, I < X < Y < Z, i.e. the 2-bit code 2 z + (x ^ z) per qubit), then
//      one thread per run of equal keys adds the run's coefficients from 0 in input order (the
//      reference sums through a matrix product, masks @ coeffs, whose order is the BLAS
//      library's: a merged duplicate can differ from it in the last bit);
//   3. force_real: the merged coefficients' real parts (symplectic.py:93-96);
//   4. group by X mask in ascending order, members in string order (symplectic.py:99-108): a
//      stable radix sort of the merged terms by X mask;
//   5. phase each coefficient by (-i)^(popcount(x & z) mod 4) (symplectic.py:110-111), written
//      with the products of NumPy's complex multiplication so that results agree bit for bit.
#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {

int scan_row_counts(int64_t *v, int64_t D, int64_t *bsum, cudaStream_t st);
size_t sort_perm_scratch(int64_t n);
int sort_perm(const uint64_t *const *words, int nw, int64_t n, int64_t *perm, void *scratch,
              cudaStream_t st);

namespace {

int grid_n(int64_t n) {
    int64_t g = (n + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

__host__ __device__ inline size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

struct TermsLayout {
    size_t fl, x1, z1, c1, klo, khi, perm, start, x2, z2, c2, perm2, flags, sort, bsum, out, total;
};

TermsLayout terms_layout(int64_t K) {
    TermsLayout L{};
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off += up256(b);
        return o;
    };
    const size_t n8 = (size_t)K * 8;
    L.fl = take(n8);
    L.x1 = take(n8);
    L.z1 = take(n8);
    L.c1 = take(2 * n8);
    L.klo = take(n8);
    L.khi = take(n8);
    L.perm = take(n8);
    L.start = take(n8 + 8);
    L.x2 = take(n8);
    L.z2 = take(n8);
    L.c2 = take(2 * n8);
    L.perm2 = take(n8);
    L.flags = take(n8);
    L.sort = take(sort_perm_scratch(K));
    L.bsum = take((size_t)((K + 1023) / 1024 + 1) * 8);
    L.out = take(64);
    L.total = off;
    return L;
}

// fl[i] = 1 when coefficient i is not zero (np.nonzero of complex values: either part)
__global__ void k_nonzero(const double2 *__restrict__ c, int64_t K, int64_t *__restrict__ fl) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < K; i += (int64_t)gridDim.x * blockDim.x)
        fl[i] = (c[i].x != 0. || c[i].y != 0.) ? 1 : 0;
}

// lexicographic key of a label: per qubit q the code 2 z + (x ^ z) (I 0, X 1, Y 2, Z 3) at bits
// 2q, 2q + 1 of a 128-bit integer (qubits 0..31 in the low word, 32..63 in the high word)
__device__ __forceinline__ uint64_t spread(uint32_t v) {  // bit k -> bit 2k
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFULL;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFULL;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0FULL;
    x = (x | (x << 2)) & 0x3333333333333333ULL;
    x = (x | (x << 1)) & 0x5555555555555555ULL;
    return x;
}

__device__ __forceinline__ uint64_t label_key(uint32_t x, uint32_t z) {
    return (spread(z) << 1) | spread(x ^ z);
}

// keep the nonzero terms in input order (fl: inclusive scan of the flags) and form their keys
__global__ void k_keep(const uint64_t *__restrict__ x, const uint64_t *__restrict__ z,
                       const double2 *__restrict__ c, int64_t K, const int64_t *__restrict__ fl,
                       uint64_t *__restrict__ x1, uint64_t *__restrict__ z1, double2 *__restrict__ c1,
                       uint64_t *__restrict__ klo, uint64_t *__restrict__ khi) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < K; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t prev = i ? fl[i - 1] : 0;
        if (fl[i] == prev) continue;
        const int64_t j = prev;
        const uint64_t xv = x[i], zv = z[i];
        x1[j] = xv;
        z1[j] = zv;
        c1[j] = c[i];
        klo[j] = label_key((uint32_t)xv, (uint32_t)zv);
        khi[j] = label_key((uint32_t)(xv >> 32), (uint32_t)(zv >> 32));
    }
}

// run starts of equal keys (or X masks) along a sorted permutation: flags, then positions
__global__ void k_run_flags(const uint64_t *__restrict__ a, const uint64_t *__restrict__ b,
                            const int64_t *__restrict__ perm, int64_t n, int64_t *__restrict__ fl) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool head = i == 0;
        if (!head) {
            const int64_t p = perm[i], q = perm[i - 1];
            head = a[p] != a[q] || (b && b[p] != b[q]);
        }
        fl[i] = head ? 1 : 0;
    }
}

__global__ void k_run_starts(const int64_t *__restrict__ incl, int64_t n, int64_t *__restrict__ start) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t prev = i ? incl[i - 1] : 0;
        if (incl[i] != prev) start[prev] = i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) start[incl[n - 1]] = n;
}

// one merged term per run: coefficients added from 0 in input order (the stable sort keeps it);
// force_real keeps the real part and records whether an imaginary part was dropped
__global__ void k_merge(const int64_t *__restrict__ start, int64_t U, const int64_t *__restrict__ perm,
                        const uint64_t *__restrict__ x1, const uint64_t *__restrict__ z1,
                        const double2 *__restrict__ c1, int force_real, uint64_t *__restrict__ x2,
                        uint64_t *__restrict__ z2, double2 *__restrict__ c2, int *dropped_imag) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < U; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = start[u], b = start[u + 1];
        double re = 0., im = 0.;
        for (int64_t k = a; k < b; ++k) {
            const double2 v = c1[perm[k]];
            re = __dadd_rn(re, v.x);
            im = __dadd_rn(im, v.y);
        }
        const int64_t first = perm[a];
        x2[u] = x1[first];
        z2[u] = z1[first];
        if (force_real) {
            if (im != 0.) atomicExch(dropped_imag, 1);
            im = 0.;
        }
        c2[u] = make_double2(re, im);
    }
}

// grouped output: member i of the X-sorted order, phased by (-i)^popcount(x & z); the group
// masks at the run starts; is_real cleared by any nonzero imaginary part
__global__ void k_phase_out(const int64_t *__restrict__ perm2, int64_t U, const int64_t *__restrict__ gincl,
                            const uint64_t *__restrict__ x2, const uint64_t *__restrict__ z2,
                            const double2 *__restrict__ c2, uint64_t *__restrict__ xout,
                            uint64_t *__restrict__ zout, double2 *__restrict__ cout,
                            int64_t *__restrict__ toff, int *not_real) {
    // phase table 1, -i, -1, i as (re, im)
    const double pr[4] = {1., 0., -1., 0.};
    const double pi[4] = {0., -1., 0., 1.};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < U; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = perm2[i];
        const uint64_t xv = x2[s], zv = z2[s];
        const int k = __popcll(xv & zv) & 3;
        const double2 c = c2[s];
        // NumPy's complex product (a + b i)(p + q i) = (a p - b q) + (a q + b p) i, each product
        // and sum rounded separately
        const double re = __dsub_rn(__dmul_rn(c.x, pr[k]), __dmul_rn(c.y, pi[k]));
        const double im = __dadd_rn(__dmul_rn(c.x, pi[k]), __dmul_rn(c.y, pr[k]));
        zout[i] = zv;
        cout[i] = make_double2(re, im);
        if (im != 0.) atomicExch(not_real, 1);
        const int64_t g = gincl[i];  // 1-based group number
        if (i == 0 || gincl[i - 1] != g) {
            xout[g - 1] = xv;
            toff[g - 1] = i;
        }
    }
}

__global__ void k_toff_end(int64_t *toff, const int64_t *gincl, int64_t U) {
    toff[U > 0 ? gincl[U - 1] : 0] = U;
}

}  // namespace
}  // namespace rq

using namespace rq;

RQ_API int rq_terms_group_scratch_size(int64_t K, size_t *bytes) {
    if (K < 1 || !bytes) return fail(RQ_E_ARG, "rq_terms_group_scratch_size: bad arguments");
    *bytes = terms_layout(K).total;
    return RQ_OK;
}

RQ_API int rq_terms_group(int64_t K, const uint64_t *xmask, const uint64_t *zmask,
                          const double *coef, int32_t force_real, uint64_t *xmask_out,
                          int64_t *toff_out, uint64_t *zmask_out, double *coef_out,
                          int64_t *J_out, int64_t *K_out, int32_t *flags_out, void *scratch,
                          void *stream) {
    if (K < 1 || !xmask || !zmask || !coef || !xmask_out || !toff_out || !zmask_out ||
        !coef_out || !J_out || !K_out || !flags_out || !scratch)
        return fail(RQ_E_ARG, "rq_terms_group: bad arguments");
    const TermsLayout L = terms_layout(K);
    char *w = static_cast<char *>(scratch);
    cudaStream_t st = as_stream(stream);
    auto at = [&](size_t off) { return w + off; };
    int64_t *fl = reinterpret_cast<int64_t *>(at(L.fl));
    uint64_t *x1 = reinterpret_cast<uint64_t *>(at(L.x1));
    uint64_t *z1 = reinterpret_cast<uint64_t *>(at(L.z1));
    double2 *c1 = reinterpret_cast<double2 *>(at(L.c1));
    uint64_t *klo = reinterpret_cast<uint64_t *>(at(L.klo));
    uint64_t *khi = reinterpret_cast<uint64_t *>(at(L.khi));
    int64_t *perm = reinterpret_cast<int64_t *>(at(L.perm));
    int64_t *start = reinterpret_cast<int64_t *>(at(L.start));
    uint64_t *x2 = reinterpret_cast<uint64_t *>(at(L.x2));
    uint64_t *z2 = reinterpret_cast<uint64_t *>(at(L.z2));
    double2 *c2 = reinterpret_cast<double2 *>(at(L.c2));
    int64_t *perm2 = reinterpret_cast<int64_t *>(at(L.perm2));
    int64_t *flags = reinterpret_cast<int64_t *>(at(L.flags));
    int64_t *bsum = reinterpret_cast<int64_t *>(at(L.bsum));
    int *out = reinterpret_cast<int *>(at(L.out));  // [0] dropped imaginary part, [1] not real
    const double2 *cin = reinterpret_cast<const double2 *>(coef);
    RQ_CUDA(cudaMemsetAsync(out, 0, 8, st));
    // 1. nonzero terms, in input order, with their label keys
    k_nonzero<<<grid_n(K), kThreads, 0, st>>>(cin, K, fl);
    RQ_TRY(scan_row_counts(fl, K, bsum, st));
    int64_t K1 = 0;
    RQ_CUDA(cudaMemcpyAsync(&K1, fl + K - 1, 8, cudaMemcpyDeviceToHost, st));
    k_keep<<<grid_n(K), kThreads, 0, st>>>(xmask, zmask, cin, K, fl, x1, z1, c1, klo, khi);
    RQ_CUDA(cudaGetLastError());
    RQ_CUDA(cudaStreamSynchronize(st));
    if (K1 == 0) {
        *J_out = 0;
        *K_out = 0;
        *flags_out = 2;  // no coefficients: real
        RQ_CUDA(cudaMemsetAsync(toff_out, 0, 8, st));
        RQ_CUDA(cudaStreamSynchronize(st));
        return RQ_OK;
    }
    // 2. merge equal labels
    const uint64_t *keyw[2] = {klo, khi};
    RQ_TRY(sort_perm(keyw, 2, K1, perm, at(L.sort), st));
    k_run_flags<<<grid_n(K1), kThreads, 0, st>>>(klo, khi, perm, K1, flags);
    RQ_TRY(scan_row_counts(flags, K1, bsum, st));
    k_run_starts<<<grid_n(K1), kThreads, 0, st>>>(flags, K1, start);
    int64_t U = 0;
    RQ_CUDA(cudaMemcpyAsync(&U, flags + K1 - 1, 8, cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    // 3. merged coefficients (real parts under force_real)
    k_merge<<<grid_n(U), kThreads, 0, st>>>(start, U, perm, x1, z1, c1, force_real ? 1 : 0, x2, z2,
                                             c2, out);
    RQ_CUDA(cudaGetLastError());
    // 4. groups by X mask, ascending; members keep the label order
    const uint64_t *xw[1] = {x2};
    RQ_TRY(sort_perm(xw, 1, U, perm2, at(L.sort), st));
    k_run_flags<<<grid_n(U), kThreads, 0, st>>>(x2, nullptr, perm2, U, flags);
    RQ_TRY(scan_row_counts(flags, U, bsum, st));
    // 5. phased output
    k_phase_out<<<grid_n(U), kThreads, 0, st>>>(perm2, U, flags, x2, z2, c2, xmask_out, zmask_out,
                                                 reinterpret_cast<double2 *>(coef_out), toff_out,
                                                 out + 1);
    k_toff_end<<<1, 1, 0, st>>>(toff_out, flags, U);
    RQ_CUDA(cudaGetLastError());
    int64_t J = 0;
    int h_out[2] = {0, 0};
    RQ_CUDA(cudaMemcpyAsync(&J, flags + U - 1, 8, cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaMemcpyAsync(h_out, out, 8, cudaMemcpyDeviceToHost, st));
    RQ_CUDA(cudaStreamSynchronize(st));
    *J_out = J;
    *K_out = U;
    *flags_out = (h_out[0] ? 1 : 0) | (h_out[1] ? 0 : 2);
    return RQ_OK;
}
