// Single-vector LOBPCG on the device (rqutils/ground_locg.py:182-471).
//
// Every step of the reference iteration is a fused pass over D-length vectors whose scalar
// inputs (inner products, norms, the Ritz pair) live in a device-resident state block, so an
// iteration never waits for the host.  Chunks of iterations are captured once into a CUDA graph
// and relaunched; each kernel first reads the state's `active` flag and returns at once after
// convergence, so a chunk may overshoot the last iteration at the cost of empty launches only.
//
// Reductions: FP64.  For 32-bit vectors each product is formed error-free in FP32 (p = a*b,
// e = fma(a, b, -p)) and summed with TwoSum per thread before the FP64 grid reduction, so the
// Gram entries carry FP64-level accuracy without FP64 arithmetic in the streaming loop.
//
// Variants: REFERENCE recomputes A x, A y and A p in every Rayleigh-Ritz step and A x' after the
// update (four matvecs), as the reference does; FAST carries A x and A y by linearity (one matvec
// per iteration) and recomputes them every `refresh` iterations and before accepting convergence.
// Mixed precision runs a 32-bit phase first and continues in the 64-bit type from its x and y.
#include <climits>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "rq_common.cuh"
#include "rq_host.h"
#include "rq_rows.cuh"

namespace rq {

int matvec_dispatch(const rq_operator_t &op, int32_t vtype, const void *x, void *y, void *scratch,
                    cudaStream_t st, const int *gate, const int *gate2);

namespace {

// ------------------------------------------------------------------------------------------
// device state
// ------------------------------------------------------------------------------------------
enum Slot {
    kIp0 = 0, kIp1 = 1, kVn = 2,                 // projection inner products, |v|^2
    kG10 = 3, kG20 = 4, kG21 = 5, kG00 = 6, kG11 = 7, kG22 = 8,  // Gram entries
    kSn = 9, kTn = 10, kUn = 11,                 // |s|^2, |t|^2, |u|^2
    kAxn = 12, kRn = 13, kMisc = 14, kMisc2 = 15,
    kSlots = 16
};

struct State {
    double2 red[kSlots];
    double2 kappa[3];
    double theta;
    double tol, tol_dim;
    double switch_rel, target_rel;
    double best_r;
    double resnorm, axnorm;
    int iter, maxiter;
    int active, converged;
    int status, phase_lo;
    int stall, refresh;
    int since_refresh, want_refresh;
    int variant, matvecs;
    int certify;  // FAST: the last convergence candidate must be confirmed by fresh products
    int guard;    // replace 0/0 breakdowns (degenerate Cardano eigenvector, |s| = 0)
    int pad_[2];
};

// ------------------------------------------------------------------------------------------
// error-free dot accumulation
// ------------------------------------------------------------------------------------------
template <typename R>
struct DotAcc;

template <>
struct DotAcc<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void prod(float a, float b) {
        const float p = a * b;
        const float e = fmaf(a, b, -p);
        float t, q;
        two_sum(s, p, t, q);
        s = t;
        c += q + e;
    }
    __device__ __forceinline__ void nprod(float a, float b) { prod(-a, b); }
    __device__ __forceinline__ double get() const { return (double)s + (double)c; }
    // the same sum as a double-float, without FP64 arithmetic
    __device__ __forceinline__ df get_df() const {
        const float h = s + c;
        return {h, c - (h - s)};
    }
};

template <>
struct DotAcc<double> {
    double s = 0.;
    __device__ __forceinline__ void prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ void nprod(double a, double b) { s = fma(-a, b, s); }
    __device__ __forceinline__ double get() const { return s; }
    __device__ __forceinline__ df get_df() const { return df_of(s); }
};

template <typename R>
struct CDot {
    DotAcc<R> re, im;
    // conj(a) * b
    __device__ __forceinline__ void add(cx<R> a, cx<R> b, bool cplx) {
        re.prod(a.re, b.re);
        if (cplx) {
            re.prod(a.im, b.im);
            im.prod(a.re, b.im);
            im.nprod(a.im, b.re);
        }
    }
    __device__ __forceinline__ double2 get() const { return make_double2(re.get(), im.get()); }
    // real vectors leave im at zero: no conversion for it
    __device__ __forceinline__ cdf get_cdf(bool cplx = true) const {
        return {re.get_df(), cplx ? im.get_df() : df{0.f, 0.f}};
    }
};

template <typename R>
__device__ __forceinline__ cx<R> axpy(cx<R> a, cx<R> x, cx<R> y) {  // a*x + y
    return {a.re * x.re - a.im * x.im + y.re, a.re * x.im + a.im * x.re + y.im};
}

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double den = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

#define GATE(st) \
    if ((st)->active == 0) return;

// ------------------------------------------------------------------------------------------
// segment policies: which rows a block handles and where its sums go
// ------------------------------------------------------------------------------------------

// Grid barrier of the persistent LOBPCG kernel (zeroed before each launch).
struct GridBar {
    unsigned int count;
    unsigned int gen;
    int abort;
    int pad_;
};

// One problem: grid-stride over [0, D), deterministic grid reduction into the state.
struct SegOne {
    State *st;
    int64_t D;
    void *red;
    __device__ __forceinline__ State *state() const { return st; }
    __device__ __forceinline__ int64_t begin() const {
        return blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    }
    __device__ __forceinline__ int64_t end() const { return D; }
    __device__ __forceinline__ int64_t stride() const { return (int64_t)gridDim.x * blockDim.x; }
    template <int NV>
    __device__ void reduce(cdf (&v)[NV], int slot) const {
        grid_reduce<NV>(v, red, st->red + slot);
    }
};

// Many problems: block c handles chunk c, rows [crow[c], crow[c + 1]) of problem cprob[c];
// problem p owns chunks [cofs[p], cofs[p + 1]).  Sums: each block writes its partials; the last
// block of a problem (per-problem counter) adds that problem's partials in chunk order.
struct SegBatch {
    State *states;
    const int32_t *cprob;
    const int64_t *crow;    // first row of each chunk
    const int64_t *cend;    // one past the last row of each chunk
    const int32_t *cofs;
    double2 *part;          // [nchunks * kMaxReduce]
    unsigned int *counter;  // [P]
    __device__ __forceinline__ State *state() const { return states + cprob[blockIdx.x]; }
    __device__ __forceinline__ int64_t begin() const { return crow[blockIdx.x] + threadIdx.x; }
    __device__ __forceinline__ int64_t end() const { return cend[blockIdx.x]; }
    __device__ __forceinline__ int64_t stride() const { return blockDim.x; }
    template <int NV>
    __device__ void reduce(cdf (&v)[NV], int slot) const {
        __shared__ cdf red[kThreads / 32][NV];
        __shared__ cdf tot[NV];
        __shared__ bool last;
        const int c = blockIdx.x, p = cprob[c];
        float4 *pt = reinterpret_cast<float4 *>(part);
        cdf w[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) w[k] = v[k];
        block_sum_all<NV>(w, tot, red);
        if (threadIdx.x < NV) {
            pt[(size_t)c * kMaxReduce + threadIdx.x] = cdf_pack(tot[threadIdx.x]);
            __threadfence();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned int n = (unsigned int)(cofs[p + 1] - cofs[p]);
            last = (atomicAdd(counter + p, 1u) == n - 1);
        }
        __syncthreads();
        if (!last) return;
        __threadfence();
        if (threadIdx.x < NV) {  // chunk order: deterministic
            cdf a = cdf_zero();
            for (int cc = cofs[p]; cc < cofs[p + 1]; ++cc)
                a = cdf_add(a, cdf_unpack(__ldcg(pt + (size_t)cc * kMaxReduce + threadIdx.x)));
            states[p].red[slot + threadIdx.x] = cdf_val(a);
        }
        if (threadIdx.x == 0) counter[p] = 0u;
    }
};

// Scalars that every thread of a block needs (square roots, quotients of the reduced sums) are
// computed once by thread 0 and shared: GB300 runs FP64 division and square roots at a small
// fraction of its FP32 rate, so per-thread copies cost more than the pass itself at D <= 2^20.
#define BLOCK_SCALARS(n, body)        \
    __shared__ double bs_[n];         \
    if (threadIdx.x == 0) {           \
        double *out = bs_;            \
        body;                         \
    }                                 \
    __syncthreads();

// The same for coefficients already converted to the pass's arithmetic type R (a double ->
// float conversion also issues on the FP64 pipe).
#define BLOCK_R(n, body)              \
    __shared__ R br_[n];              \
    if (threadIdx.x == 0) {           \
        R *out = br_;                 \
        body;                         \
    }                                 \
    __syncthreads();

#define SEG_LOOP(i) for (int64_t i = seg.begin(); i < seg.end(); i += seg.stride())

// ------------------------------------------------------------------------------------------
// vector kernels (one pass each)
// ------------------------------------------------------------------------------------------

// red[slot + k] = <a_k, b_k> for k < NP
template <typename V, int NP>
struct Pairs {
    const V *a[NP];
    const V *b[NP];
};

template <typename V, int NP, typename SEG>
__device__ __forceinline__ void d_dots(SEG seg, Pairs<V, NP> pr, int slot) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    CDot<R> acc[NP];
    SEG_LOOP(i) {
#pragma unroll
        for (int k = 0; k < NP; ++k)
            acc[k].add(VT<V>::ld(pr.a[k], i), VT<V>::ld(pr.b[k], i), VT<V>::kComplex);
    }
    cdf v[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) v[k] = acc[k].get_cdf(VT<V>::kComplex);
    seg.template reduce<NP>(v, slot);
}
template <typename V, int NP, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_dots(SEG seg, Pairs<V, NP> pr, int slot) {
    d_dots<V, NP, SEG>(seg, pr, slot);
}

// out = v * scale where scale = 1 / sqrt(red[nslot].x) (1 when that is 0); optional <x,out>, <y,out>
template <typename V, typename SEG>
__device__ __forceinline__ void d_normalize(SEG seg, const V *in, V *out, int nslot) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(1, {
        const double n = sqrt(st->red[nslot].x);
        out[0] = (R)(n == 0. ? 1. : 1. / n);
    })
    const R inv = br_[0];
    SEG_LOOP(i) {
        cx<R> v = VT<V>::ld(in, i);
        VT<V>::st(out, i, {v.re * inv, v.im * inv});
    }
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_normalize(SEG seg, const V *in, V *out, int nslot) {
    d_normalize<V, SEG>(seg, in, out, nslot);
}

// v <- v - x ip0 - y ip1 (ip from red[kIp0], red[kIp1]); red[kVn] = |v|^2
template <typename V, typename SEG>
__device__ __forceinline__ void d_sub2_norm(SEG seg, const V *x, const V *y, V *v) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(4, {
        out[0] = (R)(-st->red[kIp0].x);
        out[1] = (R)(-st->red[kIp0].y);
        out[2] = (R)(-st->red[kIp1].x);
        out[3] = (R)(-st->red[kIp1].y);
    })
    const cx<R> m0 = {br_[0], br_[1]}, m1 = {br_[2], br_[3]};
    CDot<R> nn;
    SEG_LOOP(i) {
        cx<R> w = axpy(m0, VT<V>::ld(x, i), VT<V>::ld(v, i));
        w = axpy(m1, VT<V>::ld(y, i), w);
        VT<V>::st(v, i, w);
        nn.add(w, w, VT<V>::kComplex);
    }
    cdf r[1] = {nn.get_cdf(VT<V>::kComplex)};
    seg.template reduce<1>(r, kVn);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_sub2_norm(SEG seg, const V *x, const V *y, V *v) {
    d_sub2_norm<V, SEG>(seg, x, y, v);
}

// v <- v / (|v| or 1); red[kIp0] = <x, v>, red[kIp1] = <y, v>
template <typename V, typename SEG>
__device__ __forceinline__ void d_scale_dots2(SEG seg, const V *x, const V *y, V *v, int do_scale) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(1, {
        const double n = sqrt(st->red[kVn].x);
        out[0] = (R)((!do_scale || n == 0.) ? 1. : 1. / n);
    })
    const R inv = br_[0];
    CDot<R> d0, d1;
    SEG_LOOP(i) {
        cx<R> w = VT<V>::ld(v, i);
        w = {w.re * inv, w.im * inv};
        if (do_scale) VT<V>::st(v, i, w);
        d0.add(VT<V>::ld(x, i), w, VT<V>::kComplex);
        d1.add(VT<V>::ld(y, i), w, VT<V>::kComplex);
    }
    cdf r[2] = {d0.get_cdf(VT<V>::kComplex), d1.get_cdf(VT<V>::kComplex)};
    seg.template reduce<2>(r, kIp0);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_scale_dots2(SEG seg, const V *x, const V *y, V *v, int do_scale) {
    d_scale_dots2<V, SEG>(seg, x, y, v, do_scale);
}

// p = v if |v| >= 0.99 else 0 (ground_locg.py:421)
template <typename V, typename SEG>
__device__ __forceinline__ void d_mask(SEG seg, const V *v, V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(1, { out[0] = (R)(sqrt(st->red[kVn].x) >= 0.99 ? 1. : 0.); })
    const R m = br_[0];
    SEG_LOOP(i) {
        cx<R> w = VT<V>::ld(v, i);
        VT<V>::st(p, i, {w.re * m, w.im * m});
    }
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_mask(SEG seg, const V *v, V *p) {
    d_mask<V, SEG>(seg, v, p);
}

// FAST projection in one pass, no reduction: p = m (v - d0 x - d1 y) with d0, d1 from
// red[kIp0], red[kIp1] and w = |v - d0 x - d1 y|^2 in red[kVn] (all three from the six inner
// products, d_proj_coef); m = 1 / sqrt(w), or 0 when w < thr^2 |v|^2 (v numerically inside the
// span of x, y; the role of the 0.99 cut of ground_locg.py:421), |v|^2 in red[kG10 + 5].  w comes
// from a difference of inner products, whose rounding floor is about eps |v|^2; the FP64 cut
// thr = 1e-7 (thr^2 = 1e-14) stays above that floor, so a w that is only rounding is never used
// to scale p (a wrong scale would make the Rayleigh-Ritz basis non-orthonormal).
template <typename V, typename SEG>
__device__ __forceinline__ void d_sub2_scale(SEG seg, const V *x, const V *y, const V *v, V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(5, {
        const double n2 = st->red[kVn].x;
        const double r2 = st->red[kG10 + 5].x;
        const double thr = sizeof(R) == 4 ? 1e-5 : 1e-7;
        const double m = (n2 > 0. && n2 > thr * thr * r2) ? 1. / sqrt(n2) : 0.;
        out[0] = (R)m;
        out[1] = (R)(-m * st->red[kIp0].x);
        out[2] = (R)(-m * st->red[kIp0].y);
        out[3] = (R)(-m * st->red[kIp1].x);
        out[4] = (R)(-m * st->red[kIp1].y);
    })
    const R m = br_[0];
    const cx<R> a0 = {br_[1], br_[2]}, a1 = {br_[3], br_[4]};
    SEG_LOOP(i) {
        const cx<R> vi = VT<V>::ld(v, i);
        cx<R> w = axpy(a0, VT<V>::ld(x, i), {vi.re * m, vi.im * m});
        w = axpy(a1, VT<V>::ld(y, i), w);
        VT<V>::st(p, i, w);
    }
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_sub2_scale(SEG seg, const V *x, const V *y, const V *v, V *p) {
    d_sub2_scale<V, SEG>(seg, x, y, v, p);
}

// Gram entries of (x, y, p): <y,Ax> <p,Ax> <p,Ay> <x,Ax> <y,Ay> <p,Ap>
template <typename V, typename SEG>
__device__ __forceinline__ void d_gram3(SEG seg, const V *x, const V *y, const V *p, const V *ax, const V *ay,
        const V *ap) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    CDot<R> g[6];
    const bool c = VT<V>::kComplex;
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i), yi = VT<V>::ld(y, i), pi = VT<V>::ld(p, i);
        const cx<R> axi = VT<V>::ld(ax, i), ayi = VT<V>::ld(ay, i), api = VT<V>::ld(ap, i);
        g[0].add(yi, axi, c);
        g[1].add(pi, axi, c);
        g[2].add(pi, ayi, c);
        g[3].add(xi, axi, c);
        g[4].add(yi, ayi, c);
        g[5].add(pi, api, c);
    }
    cdf r[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) r[k] = g[k].get_cdf(VT<V>::kComplex);
    seg.template reduce<6>(r, kG10);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_gram3(SEG seg, const V *x, const V *y, const V *p, const V *ax, const V *ay,
        const V *ap) {
    d_gram3<V, SEG>(seg, x, y, p, ax, ay, ap);
}

// Gram entries of (x, p) for the first Rayleigh-Ritz step: <p,Ax> <x,Ax> <p,Ap>
template <typename V, typename SEG>
__device__ __forceinline__ void d_gram2(SEG seg, const V *x, const V *p, const V *ax, const V *ap) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    CDot<R> g[3];
    const bool c = VT<V>::kComplex;
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i), pi = VT<V>::ld(p, i);
        const cx<R> axi = VT<V>::ld(ax, i), api = VT<V>::ld(ap, i);
        g[0].add(pi, axi, c);
        g[1].add(xi, axi, c);
        g[2].add(pi, api, c);
    }
    cdf r[3] = {g[0].get_cdf(VT<V>::kComplex), g[1].get_cdf(VT<V>::kComplex), g[2].get_cdf(VT<V>::kComplex)};
    seg.template reduce<3>(r, kG10);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_gram2(SEG seg, const V *x, const V *p, const V *ax, const V *ap) {
    d_gram2<V, SEG>(seg, x, p, ax, ap);
}

// s = k1 y + k2 p: red[kSn] = |s|^2
template <typename V, typename SEG>
__device__ __forceinline__ void d_upd_s(SEG seg, const V *y, const V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(4, {
        out[0] = (R)st->kappa[1].x;
        out[1] = (R)st->kappa[1].y;
        out[2] = (R)st->kappa[2].x;
        out[3] = (R)st->kappa[2].y;
    })
    const cx<R> k1 = {br_[0], br_[1]}, k2 = {br_[2], br_[3]};
    CDot<R> nn;
    SEG_LOOP(i) {
        const cx<R> s = axpy(k2, VT<V>::ld(p, i), cmul(k1, VT<V>::ld(y, i)));
        nn.add(s, s, VT<V>::kComplex);
    }
    cdf r[1] = {nn.get_cdf(VT<V>::kComplex)};
    seg.template reduce<1>(r, kSn);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_upd_s(SEG seg, const V *y, const V *p) {
    d_upd_s<V, SEG>(seg, y, p);
}

// t = s (k0/|s|) - x |s|, u = k0 x + s: red[kTn] = |t|^2, red[kUn] = |u|^2
template <typename V, typename SEG>
__device__ __forceinline__ void d_upd_tu(SEG seg, const V *x, const V *y, const V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(10, {
        const double ns = sqrt(st->red[kSn].x);
        out[0] = (R)(-ns);
        out[1] = (R)(st->kappa[0].x / ns);
        out[2] = (R)(st->kappa[0].y / ns);
        out[3] = (R)st->kappa[0].x;
        out[4] = (R)st->kappa[0].y;
        out[5] = (R)st->kappa[1].x;
        out[6] = (R)st->kappa[1].y;
        out[7] = (R)st->kappa[2].x;
        out[8] = (R)st->kappa[2].y;
        out[9] = (R)((st->guard && ns == 0.) ? 1 : 0);  // s = 0: y' = y instead of 0 * inf
    })
    const bool keep_y = br_[9] != (R)0;
    const cx<R> k0 = {br_[3], br_[4]}, k1 = {br_[5], br_[6]}, k2 = {br_[7], br_[8]};
    const cx<R> k0s = {br_[1], br_[2]};
    const cx<R> mns = {br_[0], (R)0};
    CDot<R> tn, un;
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i);
        const cx<R> s = axpy(k2, VT<V>::ld(p, i), cmul(k1, VT<V>::ld(y, i)));
        const cx<R> t = keep_y ? VT<V>::ld(y, i) : axpy(mns, xi, cmul(k0s, s));
        const cx<R> u = axpy(k0, xi, s);
        tn.add(t, t, VT<V>::kComplex);
        un.add(u, u, VT<V>::kComplex);
    }
    cdf r[2] = {tn.get_cdf(VT<V>::kComplex), un.get_cdf(VT<V>::kComplex)};
    seg.template reduce<2>(r, kTn);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_upd_tu(SEG seg, const V *x, const V *y, const V *p) {
    d_upd_tu<V, SEG>(seg, x, y, p);
}

// FAST: s = k1 y + k2 p once, with <s,s>, <x,s>, <x,x>, <y,y> into kG10..kG10+3 (the norms of
// t = s k0/|s| - x |s| and u = k0 x + s follow from them, d_stu_coef), one reduction instead of two
template <typename V, typename SEG>
__device__ __forceinline__ void d_upd_stu(SEG seg, const V *x, const V *y, const V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(4, {
        out[0] = (R)st->kappa[1].x;
        out[1] = (R)st->kappa[1].y;
        out[2] = (R)st->kappa[2].x;
        out[3] = (R)st->kappa[2].y;
    })
    const cx<R> k1 = {br_[0], br_[1]}, k2 = {br_[2], br_[3]};
    CDot<R> ss, xs, xx, yy;
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i), yi = VT<V>::ld(y, i);
        const cx<R> si = axpy(k2, VT<V>::ld(p, i), cmul(k1, yi));
        ss.add(si, si, VT<V>::kComplex);
        xs.add(xi, si, VT<V>::kComplex);
        xx.add(xi, xi, VT<V>::kComplex);
        yy.add(yi, yi, VT<V>::kComplex);
    }
    cdf r[4] = {ss.get_cdf(VT<V>::kComplex), xs.get_cdf(VT<V>::kComplex), xx.get_cdf(VT<V>::kComplex),
                yy.get_cdf(VT<V>::kComplex)};
    seg.template reduce<4>(r, kG10);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads) k_upd_stu(SEG seg, const V *x, const V *y, const V *p) {
    d_upd_stu<V, SEG>(seg, x, y, p);
}

// x <- u / |u|, y <- t / |t|; FAST also carries A x, A y by the same combinations.
template <typename V, bool CARRY, typename SEG>
__device__ __forceinline__ void d_upd_xy(SEG seg, V *x, V *y, const V *p, V *ax, V *ay, const V *ap) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(12, {
        const double ns = sqrt(st->red[kSn].x);
        out[0] = (R)(-ns);
        out[1] = (R)(st->kappa[0].x / ns);
        out[2] = (R)(st->kappa[0].y / ns);
        out[3] = (R)st->kappa[0].x;
        out[4] = (R)st->kappa[0].y;
        out[5] = (R)st->kappa[1].x;
        out[6] = (R)st->kappa[1].y;
        out[7] = (R)st->kappa[2].x;
        out[8] = (R)st->kappa[2].y;
        out[9] = (R)((st->guard && ns == 0.) ? 1 : 0);  // s = 0: y' = y instead of 0 * inf
        out[10] = (R)(1. / sqrt(st->red[kTn].x));
        out[11] = (R)(1. / sqrt(st->red[kUn].x));
    })
    const bool keep_y = br_[9] != (R)0;
    const cx<R> k0 = {br_[3], br_[4]}, k1 = {br_[5], br_[6]}, k2 = {br_[7], br_[8]};
    const cx<R> k0s = {br_[1], br_[2]};
    const cx<R> mns = {br_[0], (R)0};
    const R rit = br_[10], riu = br_[11];
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i);
        const cx<R> yi = VT<V>::ld(y, i);
        const cx<R> s = axpy(k2, VT<V>::ld(p, i), cmul(k1, yi));
        const cx<R> t = keep_y ? yi : axpy(mns, xi, cmul(k0s, s));
        const cx<R> u = axpy(k0, xi, s);
        VT<V>::st(x, i, {u.re * riu, u.im * riu});
        VT<V>::st(y, i, {t.re * rit, t.im * rit});
        if (CARRY) {
            const cx<R> axi = VT<V>::ld(ax, i);
            const cx<R> ayi = VT<V>::ld(ay, i);
            const cx<R> as = axpy(k2, VT<V>::ld(ap, i), cmul(k1, ayi));
            const cx<R> at = keep_y ? ayi : axpy(mns, axi, cmul(k0s, as));
            const cx<R> au = axpy(k0, axi, as);
            VT<V>::st(ax, i, {au.re * riu, au.im * riu});
            VT<V>::st(ay, i, {at.re * rit, at.im * rit});
        }
    }
}
template <typename V, bool CARRY, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_upd_xy(SEG seg, V *x, V *y, const V *p, V *ax, V *ay, const V *ap) {
    d_upd_xy<V, CARRY, SEG>(seg, x, y, p, ax, ay, ap);
}

// iteration 1 update (ground_locg.py:278-281): t = p k0 - x k1, u = x k0 + p k1 -> norms
template <typename V, typename SEG>
__device__ __forceinline__ void d_upd2_norms(SEG seg, const V *x, const V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(4, {
        out[0] = (R)st->kappa[0].x;
        out[1] = (R)st->kappa[0].y;
        out[2] = (R)st->kappa[1].x;
        out[3] = (R)st->kappa[1].y;
    })
    const cx<R> k0 = {br_[0], br_[1]}, k1 = {br_[2], br_[3]};
    const cx<R> mk1 = {-k1.re, -k1.im};
    CDot<R> tn, un;
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i), pi = VT<V>::ld(p, i);
        const cx<R> t = axpy(mk1, xi, cmul(k0, pi));
        const cx<R> u = axpy(k1, pi, cmul(k0, xi));
        tn.add(t, t, VT<V>::kComplex);
        un.add(u, u, VT<V>::kComplex);
    }
    cdf r[2] = {tn.get_cdf(VT<V>::kComplex), un.get_cdf(VT<V>::kComplex)};
    seg.template reduce<2>(r, kTn);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_upd2_norms(SEG seg, const V *x, const V *p) {
    d_upd2_norms<V, SEG>(seg, x, p);
}

template <typename V, typename SEG>
__device__ __forceinline__ void d_upd2_xy(SEG seg, V *x, V *y, const V *p) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(6, {
        out[0] = (R)st->kappa[0].x;
        out[1] = (R)st->kappa[0].y;
        out[2] = (R)st->kappa[1].x;
        out[3] = (R)st->kappa[1].y;
        out[4] = (R)(1. / sqrt(st->red[kTn].x));
        out[5] = (R)(1. / sqrt(st->red[kUn].x));
    })
    const cx<R> k0 = {br_[0], br_[1]}, k1 = {br_[2], br_[3]};
    const cx<R> mk1 = {-k1.re, -k1.im};
    const R rit = br_[4], riu = br_[5];
    SEG_LOOP(i) {
        const cx<R> xi = VT<V>::ld(x, i), pi = VT<V>::ld(p, i);
        const cx<R> t = axpy(mk1, xi, cmul(k0, pi));
        const cx<R> u = axpy(k1, pi, cmul(k0, xi));
        VT<V>::st(x, i, {u.re * riu, u.im * riu});
        VT<V>::st(y, i, {t.re * rit, t.im * rit});
    }
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_upd2_xy(SEG seg, V *x, V *y, const V *p) {
    d_upd2_xy<V, SEG>(seg, x, y, p);
}

// r = Ax - theta x; red[kAxn] = |Ax|^2, red[kRn] = |r|^2.  theta from st->theta, or from
// Re red[kMisc] (iteration 0: rho = Re <x, Ax>) when use_rho.
template <typename V, typename SEG>
__device__ __forceinline__ void d_resid(SEG seg, const V *ax, const V *x, V *r, int use_rho) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    BLOCK_R(1, { out[0] = (R)(-(use_rho ? st->red[kMisc].x : st->theta)); })
    const cx<R> mth = {br_[0], (R)0};
    CDot<R> an, rn;
    SEG_LOOP(i) {
        const cx<R> a = VT<V>::ld(ax, i);
        const cx<R> w = axpy(mth, VT<V>::ld(x, i), a);
        VT<V>::st(r, i, w);
        an.add(a, a, VT<V>::kComplex);
        rn.add(w, w, VT<V>::kComplex);
    }
    cdf out[2] = {an.get_cdf(VT<V>::kComplex), rn.get_cdf(VT<V>::kComplex)};
    seg.template reduce<2>(out, kAxn);
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_resid(SEG seg, const V *ax, const V *x, V *r, int use_rho) {
    d_resid<V, SEG>(seg, ax, x, r, use_rho);
}

// w = r / (d - theta), |d - theta| floored at 1e-8 (1 + |theta|): the Jacobi preconditioner.
template <typename V, typename SEG>
__device__ __forceinline__ void d_jacobi(SEG seg, const double *diag, const V *r, V *w) {
    State *st = seg.state();
    GATE(st);
    using R = typename VT<V>::R;
    // a preconditioner needs no FP64 quotient: the reciprocal is taken in FP32 (GB300's FP64
    // division costs more than the rest of the pass)
    __shared__ double th_s;
    __shared__ float floor_s;
    if (threadIdx.x == 0) {
        th_s = st->theta;
        floor_s = (float)(1e-8 * (1. + fabs(st->theta)));
    }
    __syncthreads();
    const double th = th_s;
    const float floor_ = floor_s;
    SEG_LOOP(i) {
        float den = (float)(diag[i] - th);
        if (fabsf(den) < floor_) den = den < 0.f ? -floor_ : floor_;
        const R f = (R)(1.f / den);
        const cx<R> v = VT<V>::ld(r, i);
        VT<V>::st(w, i, {v.re * f, v.im * f});
    }
}
template <typename V, typename SEG>
__global__ void __launch_bounds__(kThreads)
k_jacobi(SEG seg, const double *diag, const V *r, V *w) {
    d_jacobi<V, SEG>(seg, diag, r, w);
}

template <typename VS, typename VD>
__global__ void __launch_bounds__(kThreads) k_convert(int64_t D, const VS *a, VD *b) {
    using RS = typename VT<VS>::R;
    using RD = typename VT<VD>::R;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const cx<RS> v = VT<VS>::ld(a, i);
        VT<VD>::st(b, i, {(RD)v.re, (RD)v.im});
    }
}

// ------------------------------------------------------------------------------------------
// scalar kernels: one thread per problem
// ------------------------------------------------------------------------------------------
// scalar steps: problem p_ = first, first + step, ... (one thread per problem in the kernels; the
// persistent kernel runs them on thread 0 of every block, on the block's own copy of the state)
#define FOR_ACTIVE_PROBLEMS(states, P, st)                                          \
    for (int p_ = first; p_ < (P); p_ += step)                                     \
        for (State *st = (states) + p_; st != nullptr && st->active; st = nullptr)

// Lowest eigenpair of a Hermitian 3x3 given by its strict lower triangle (m10, m20, m21) and its
// diagonal (complex values, real part used as in ground_locg.py:446); Cardano (Kopp 2008).
// Smallest root of lambda^3 + c2 lambda^2 + c1 lambda + c0 (three real roots) without FP64
// transcendental functions: the trigonometric (Cardano) root in FP32 as a seed, then Newton steps
// on the cubic in FP64 (the reciprocal of f' from an FP32 estimate and one FP64 correction).
// When the two lowest roots lie within the seed's error Newton may settle on the upper one, so
// the quotient quadratic lambda^2 + (c2 + x) lambda + c1 + x (c2 + x) gives the other two roots
// and a smaller one replaces x (random Hermitian 3x3: within 3e-15 of the largest eigenvalue's
// magnitude; nearly double lowest roots: within 1.6e-8, the FP64 trigonometric formula 2.4e-8).
// Returns false when the steps do not settle to the FP64 rounding level: the caller then takes
// the FP64 trigonometric root.
__device__ __forceinline__ bool cubic_min_root_fast(double c2, double c1, double c0, double p,
                                                   double q, double disc, double &lam) {
    // atan2 is scale-free: scale both arguments into FP32 range first
    const double yd = sqrt(fmax(disc, 0.)), sc = fmax(fabs(yd), fabs(q));
    if (!(sc > 0.) || !isfinite(sc) || !(p > 0.)) return false;
    const double isc = 1. / sc;
    const float phi = atan2f((float)(yd * isc), (float)(q * isc)) * (1.f / 3.f);
    float cp, sp;
    sincosf(phi, &sp, &cp);
    const float s3 = 1.7320508f;
    const float xmin = fminf(2.f * cp, fminf(-cp - s3 * sp, -cp + s3 * sp));
    const double sqp = (double)sqrtf((float)p);
    double x = sqp * (1. / 3.) * (double)xmin - c2 * (1. / 3.);
    const double tol = 4e-16 * (fabs(x) + sqp);
    for (int it = 0; it < 4; ++it) {
        const double f = fma(fma(x + c2, x, c1), x, c0);
        const double fp = fma(fma(3., x, 2. * c2), x, c1);
        double r = (double)(1.f / (float)fp);
        r = r * fma(-fp, r, 2.);  // one Newton step on the reciprocal: ~1e-14 relative
        const double dx = f * r;
        x -= dx;
        if (!isfinite(x)) return false;
        if (fabs(dx) <= tol) {
            const double b = c2 + x, c = fma(x, b, c1), d2 = fma(b, b, -4. * c);
            if (d2 > 0.) {
                const double rm = (-b - sqrt(d2)) * 0.5;
                if (rm < x) x = rm;
            }
            lam = x;
            return true;
        }
    }
    return false;
}

__device__ void eig3(double2 m10, double2 m20, double2 m21, double2 m00, double2 m11, double2 m22,
                     double &lam, double2 (&v)[3], bool guard = false, bool fast = false) {
    const double d0 = m00.x, d1 = m11.x, d2 = m22.x;
    const double a10 = m10.x * m10.x + m10.y * m10.y;
    const double a20 = m20.x * m20.x + m20.y * m20.y;
    const double a21 = m21.x * m21.x + m21.y * m21.y;
    const double c2 = -(d0 + d1 + d2);
    const double c1 = (d0 * d2 + d1 * d0 + d2 * d1) - (a10 + a20 + a21);
    double c0 = d0 * a21 + d1 * a20 + d2 * a10;
    c0 -= d0 * d1 * d2;
    // Re(m02 m10 m21) with m02 = conj(m20)
    const double2 m02 = make_double2(m20.x, -m20.y);
    const double2 t = make_double2(m02.x * m10.x - m02.y * m10.y, m02.x * m10.y + m02.y * m10.x);
    c0 -= 2. * (t.x * m21.x - t.y * m21.y);
    const double p = c2 * c2 - 3. * c1;
    const double q = -13.5 * c0 - c2 * c2 * c2 + 4.5 * c2 * c1;
    // divisions by 3 as products with 1/3 (GB300 runs an FP64 division as a long FP64 sequence
    // on one thread here; the results differ from the quotients by at most an ulp)
    constexpr double kThird = 1. / 3.;
    const double disc = 27. * (0.25 * c1 * c1 * (p - c1) + c0 * (q + 6.75 * c0));
    if (!(fast && cubic_min_root_fast(c2, c1, c0, p, q, disc, lam))) {
        const double phi = atan2(sqrt(disc), q) * kThird;
        const double cp = cos(phi), sp = sin(phi), s3 = sqrt(3.);
        double xmin = 2. * cp;
        xmin = fmin(xmin, -cp - s3 * sp);
        xmin = fmin(xmin, -cp + s3 * sp);
        if (isnan(cp) || isnan(sp)) xmin = NAN;  // jnp.min propagates NaN
        lam = sqrt(p) * kThird * xmin - c2 * kThird;
    }
    // columns 1 and 2 of (A - lambda I): a = (m01, m11 - l, m21), b = (m02, m12, m22 - l)
    const double2 a0 = make_double2(m10.x, -m10.y), a1 = make_double2(m11.x - lam, m11.y), a2 = m21;
    const double2 b0 = m02, b1 = make_double2(m21.x, -m21.y), b2 = make_double2(m22.x - lam, m22.y);
    auto mul = [](double2 u, double2 w) {
        return make_double2(u.x * w.x - u.y * w.y, u.x * w.y + u.y * w.x);
    };
    auto sub = [](double2 u, double2 w) { return make_double2(u.x - w.x, u.y - w.y); };
    double2 c[3] = {sub(mul(a1, b2), mul(a2, b1)), sub(mul(a2, b0), mul(a0, b2)),
                    sub(mul(a0, b1), mul(a1, b0))};
    double nrm = 0.;
    for (int k = 0; k < 3; ++k) {
        c[k].y = -c[k].y;  // conjugate
        nrm += c[k].x * c[k].x + c[k].y * c[k].y;
    }
    nrm = sqrt(nrm);
    if (guard && !(nrm > 0. && isfinite(nrm)) && isfinite(lam)) {
        // columns 1 and 2 of (A - lambda I) are parallel (or zero): the eigenvector is
        // orthogonal to the other column pairs; take the larger of their cross products
        const double2 z0 = make_double2(m00.x - lam, m00.y);
        const double2 col0[3] = {z0, m10, m20};
        const double2 col1[3] = {a0, a1, a2};
        const double2 col2[3] = {b0, b1, b2};
        double best = 0.;
        for (int pair = 0; pair < 2; ++pair) {
            const double2 *u = col0, *w = pair == 0 ? col1 : col2;
            double2 e[3] = {sub(mul(u[1], w[2]), mul(u[2], w[1])), sub(mul(u[2], w[0]), mul(u[0], w[2])),
                            sub(mul(u[0], w[1]), mul(u[1], w[0]))};
            double n2 = 0.;
            for (int k = 0; k < 3; ++k) {
                e[k].y = -e[k].y;
                n2 += e[k].x * e[k].x + e[k].y * e[k].y;
            }
            if (n2 > best && isfinite(n2)) {
                best = n2;
                for (int k = 0; k < 3; ++k) c[k] = e[k];
            }
        }
        nrm = sqrt(best);
        if (!(nrm > 0.)) {  // A = lambda I on the span: any vector; keep x
            c[0] = make_double2(1., 0.);
            c[1] = c[2] = make_double2(0., 0.);
            nrm = 1.;
        }
    }
    const double inv = 1. / nrm;
    for (int k = 0; k < 3; ++k) v[k] = make_double2(c[k].x * inv, c[k].y * inv);
}

__device__ __forceinline__ void d_rr3(State *states, int P, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
        double lam;
        double2 v[3];
        // FAST: the Newton-polished root (no FP64 atan2 / cos / sin on the solve's one thread)
        eig3(st->red[kG10], st->red[kG20], st->red[kG21], st->red[kG00], st->red[kG11],
             st->red[kG22], lam, v, st->guard != 0, st->variant == RQ_LOBPCG_FAST);
        st->theta = lam;
        for (int k = 0; k < 3; ++k) st->kappa[k] = v[k];
        break;
    }
}
__global__ void k_rr3(State *states, int P) { d_rr3(states, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x); }

// eigenpair_2x2 (ground_locg.py:424-435) of [[g00, conj(g10)], [g10, g11]]
__device__ __forceinline__ void d_rr2(State *states, int P, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
    // k_gram2 wrote <p,Ax>, <x,Ax>, <p,Ap> to three consecutive slots from kG10
    const double2 m10 = st->red[kG10];
    const double d0 = st->red[kG10 + 1].x;  // <x, Ax>
    const double d1 = st->red[kG10 + 2].x;  // <p, Ap>
    const double det = d0 * d1 - (m10.x * m10.x + m10.y * m10.y);
    const double tr = d0 + d1;
    const double lam = (tr - sqrt(tr * tr - 4. * det)) * 0.5;
    const double2 num = make_double2(d1 - lam + m10.x, -m10.y);
    const double2 den = make_double2(d0 - lam + m10.x, m10.y);
    double2 v0 = cdiv(num, den);
    const double n = sqrt(v0.x * v0.x + v0.y * v0.y + 1.);
    st->theta = lam;
    st->kappa[0] = make_double2(v0.x / n, v0.y / n);
    st->kappa[1] = make_double2(-1. / n, 0.);
    st->kappa[2] = make_double2(0., 0.);
    break;
    }
}
__global__ void k_rr2(State *states, int P) { d_rr2(states, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x); }

// red[slot] = 0 for the active problems
__global__ void k_clear_slot(State *states, int P, int slot) {
    const int first = blockIdx.x * blockDim.x + threadIdx.x, step = gridDim.x * blockDim.x;
    FOR_ACTIVE_PROBLEMS(states, P, st) {
    st->red[slot] = make_double2(0., 0.);
    break;
    }
}

// iteration 0: rho = Re <x, Ax> into red[kMisc] (already there from k_dots); nothing else.

// Convergence test of ground_locg.py:329-334 and phase bookkeeping; a problem that stops
// decrements the count of active problems.
__device__ __forceinline__ void d_check(State *states, int P, int *nactive, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
    const double rn = sqrt(st->red[kRn].x);
    const double an = sqrt(st->red[kAxn].x);
    const double th = st->theta;
    st->resnorm = rn;
    st->axnorm = an;
    st->iter += 1;
    ++st->since_refresh;
    bool conv;
    if (st->phase_lo) {
        // 32-bit phase: hand over once the residual is small or stops improving (the reference
        // test with the 32-bit epsilon times the dimension is meaningless for large D)
        conv = rn < st->switch_rel * fabs(th);
        if (rn < 0.7 * st->best_r) {
            st->best_r = rn;
            st->stall = 0;
        } else if (++st->stall >= 30) {
            conv = true;
        }
    } else {
        conv = rn < st->tol * ((an - th) * st->tol_dim * 10.);
        if (st->target_rel > 0. && rn <= st->target_rel * fabs(th)) conv = true;
    }
    if (!isfinite(rn) || !isfinite(th)) st->status = RQ_E_NONFINITE;
    if (st->variant == RQ_LOBPCG_FAST) {
        // carried products: confirm with fresh A x, A y before accepting
        if (conv && !st->certify) {
            st->want_refresh = 1;
            st->certify = 1;
            conv = false;
        } else if (conv) {
            st->certify = 0;
        } else {
            st->certify = 0;
            st->want_refresh = (st->since_refresh >= st->refresh) ? 1 : 0;
        }
    }
    st->converged = conv ? 1 : 0;
    if (conv || st->iter >= st->maxiter) {
        st->active = 0;
        if (nactive) atomicSub(nactive, 1);
    }
    break;
    }
}
__global__ void k_check(State *states, int P, int *nactive) {
    d_check(states, P, nactive, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// FAST: a refresh starts -- reset the counter (runs only when want_refresh is set)
// FAST projection: both rounds of classical Gram-Schmidt against (x, y) from one set of inner
// products.  With c = (<x,r>, <y,r>) and G the Gram matrix of (x, y), the second round's
// coefficients are c - G c, so r is projected once with e = 2 c - G c (slots kG10..: <x,r>, <y,r>,
// <x,x>, <x,y>, <y,y>, <r,r>; e goes to kIp0, kIp1 for the subtraction pass).
__device__ __forceinline__ void d_proj_coef(State *states, int P, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
        const double2 cx_ = st->red[kG10], cy = st->red[kG10 + 1];
        const double2 gxx = st->red[kG10 + 2], gxy = st->red[kG10 + 3], gyy = st->red[kG10 + 4];
        auto mul = [](double2 a, double2 b) {
            return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
        };
        const double2 gyx = make_double2(gxy.x, -gxy.y);  // <y, x>
        const double2 ax = mul(gxx, cx_), bx = mul(gxy, cy);
        const double2 ay = mul(gyx, cx_), by = mul(gyy, cy);
        const double2 d0 = make_double2(2. * cx_.x - ax.x - bx.x, 2. * cx_.y - ax.y - bx.y);
        const double2 d1 = make_double2(2. * cy.x - ay.x - by.x, 2. * cy.y - ay.y - by.y);
        st->red[kIp0] = d0;
        st->red[kIp1] = d1;
        // |r - d0 x - d1 y|^2 = <r,r> - 2 Re(conj(d0) <x,r> + conj(d1) <y,r>) + |d0|^2 <x,x>
        //                       + |d1|^2 <y,y> + 2 Re(conj(d0) d1 <x,y>)
        const double2 d0c = make_double2(d0.x, -d0.y), d1c = make_double2(d1.x, -d1.y);
        const double2 d01 = mul(d0c, d1);
        const double n2 = st->red[kG10 + 5].x - 2. * (mul(d0c, cx_).x + mul(d1c, cy).x) +
                          (d0.x * d0.x + d0.y * d0.y) * gxx.x + (d1.x * d1.x + d1.y * d1.y) * gyy.x +
                          2. * mul(d01, gxy).x;
        st->red[kVn] = make_double2(n2, 0.);
        break;
    }
}
__global__ void k_proj_coef(State *states, int P) {
    d_proj_coef(states, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// |s|^2, |t|^2, |u|^2 of the update from <s,s>, <x,s>, <x,x>, <y,y> (d_upd_stu):
// |t|^2 = |a|^2 <s,s> + b^2 <x,x> - 2 b Re(a <x,s>) with a = k0 / |s|, b = |s| (t = y when s = 0
// under the guard), |u|^2 = |k0|^2 <x,x> + <s,s> + 2 Re(conj(k0) <x,s>)
__device__ __forceinline__ void d_stu_coef(State *states, int P, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
        const double ss = st->red[kG10].x, xx = st->red[kG10 + 2].x, yy = st->red[kG10 + 3].x;
        const double2 xs = st->red[kG10 + 1], k0 = st->kappa[0];
        const double ns = sqrt(ss);
        const double2 a = make_double2(k0.x / ns, k0.y / ns);
        const double re_axs = a.x * xs.x - a.y * xs.y;        // Re(a <x,s>)
        const double re_k0xs = k0.x * xs.x + k0.y * xs.y;     // Re(conj(k0) <x,s>)
        const double tn = (st->guard && ns == 0.) ? yy : (a.x * a.x + a.y * a.y) * ss + ss * xx - 2. * ns * re_axs;
        st->red[kSn] = make_double2(ss, 0.);
        st->red[kTn] = make_double2(tn, 0.);
        st->red[kUn] = make_double2((k0.x * k0.x + k0.y * k0.y) * xx + ss + 2. * re_k0xs, 0.);
        break;
    }
}
__global__ void k_stu_coef(State *states, int P) {
    d_stu_coef(states, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__device__ __forceinline__ void d_refresh_mark(State *states, int P, int first, int step) {
    FOR_ACTIVE_PROBLEMS(states, P, st) {
        if (st->want_refresh) {
            st->since_refresh = 0;
            st->matvecs += 2;
        }
        break;
    }
}
__global__ void k_refresh_mark(State *states, int P) {
    d_refresh_mark(states, P, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ------------------------------------------------------------------------------------------
// host driver
// ------------------------------------------------------------------------------------------
constexpr int kChunk = 8;  // iterations per captured graph (1 with a matvec callback)

struct Layout {
    size_t state, red, err, vec_lo, vec_hi, total;
    int64_t D;
    size_t lo_bytes, hi_bytes;
};

int lo_type(int32_t hi) {
    switch (hi) {
        case RQ_F64: return RQ_F32;
        case RQ_C128: return RQ_C64;
        default: return hi;
    }
}

Layout layout(int64_t D, const rq_lobpcg_params_t &p) {
    Layout L{};
    L.D = D;
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t o = off;
        off += (b + 255) & ~size_t(255);
        return o;
    };
    L.state = take(sizeof(State));
    L.err = take(64);  // [0] matvec error flag, [8] active count, [16] grid barrier
    L.red = take(reduce_scratch_bytes());
    L.hi_bytes = (size_t)D * vtype_size(p.vtype);
    L.lo_bytes = (size_t)D * vtype_size(lo_type(p.vtype));
    L.vec_hi = take(8 * ((L.hi_bytes + 255) & ~size_t(255)));
    L.vec_lo = p.mixed ? take(8 * ((L.lo_bytes + 255) & ~size_t(255))) : 0;
    L.total = off;
    return L;
}

int grid_vec(int64_t D) {
    int64_t g = (D + kThreads - 1) / kThreads;
    const int64_t cap = (int64_t)sm_count() * 4;
    if (g > cap) g = cap;
    if (g > kMaxReduceBlocks) g = kMaxReduceBlocks;
    return (int)(g < 1 ? 1 : g);
}

// Vectors of one phase: x, y, r, p, Ax, Ay, Ap, w.
template <typename V>
struct Vecs {
    V *x, *y, *r, *p, *ax, *ay, *ap, *w;
};

template <typename V>
Vecs<V> carve_vecs(char *base, size_t bytes) {
    const size_t s = (bytes + 255) & ~size_t(255);
    Vecs<V> v;
    V **ptr[8] = {&v.x, &v.y, &v.r, &v.p, &v.ax, &v.ay, &v.ap, &v.w};
    for (int k = 0; k < 8; ++k) *ptr[k] = reinterpret_cast<V *>(base + k * s);
    return v;
}

// Matvec of a phase: the operator's own kernels gated by the problem's flags, or a caller
// callback.  `refresh` marks the FAST variant's gated recomputation of A x, A y.
struct MvOne {
    const rq_operator_t *op;
    void *scratch;
    int operator()(int32_t vt, const void *in, void *out, cudaStream_t s, State *states,
                   bool refresh) const {
        return matvec_dispatch(*op, vt, in, out, scratch, s, &states->active,
                               refresh ? &states->want_refresh : nullptr);
    }
};

struct MvCallback {
    rq_matvec_fn fn;
    void *ctx;
    int operator()(int32_t vt, const void *in, void *out, cudaStream_t s, State *,
                   bool refresh) const {
        if (refresh) return RQ_OK;  // callbacks run the REFERENCE variant
        const int rc = fn(ctx, vt, in, out, s);
        return rc == 0 ? RQ_OK : fail(RQ_E_ARG, "rq_lobpcg_solve_cb: the matvec callback failed");
    }
};

struct BatchPersist;  // the persistent batched solve's plan (below)

template <typename V, typename SEG, typename MV>
struct Phase {
    MV mv;
    int32_t vtype;
    SEG seg;
    int grid;
    State *states;
    int P;
    int *nactive;
    Vecs<V> v;
    bool jacobi;
    const double *diag;
    // set when the loop may run as one persistent cooperative kernel (one problem, cached
    // connectivity or CSR operator of this phase's value type)
    const rq_operator_t *pop = nullptr;
    GridBar *bar = nullptr;
    // set when a batched loop may run as persistent launches (cached-connectivity batches)
    BatchPersist *bp = nullptr;
    // optional: shrink the block list to the problems still active (active > 0) or restore the
    // full list (active < 0); sets `grid`
    int (*compact)(void *ctx, int active, int *grid, cudaStream_t s) = nullptr;
    void *compact_ctx = nullptr;

    int pgrid() const { return (P + 127) / 128; }

    int matvec(const V *in, V *out, cudaStream_t s, bool refresh = false) {
        return mv(vtype, in, out, s, states, refresh);
    }

    // project_out((x, y), src) -> p  (ground_locg.py:380-421); src is overwritten
    void project(V *src, cudaStream_t s, int variant = RQ_LOBPCG_REFERENCE) {
        if (variant == RQ_LOBPCG_FAST) {
            Pairs<V, 6> g{{v.x, v.y, v.x, v.x, v.y, src}, {src, src, v.x, v.y, v.y, src}};
            k_dots<V, 6, SEG><<<grid, kThreads, 0, s>>>(seg, g, kG10);
            k_proj_coef<<<pgrid(), 128, 0, s>>>(states, P);
            k_sub2_scale<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src, v.p);
            return;
        }
        Pairs<V, 2> pr{{v.x, v.y}, {src, src}};
        k_dots<V, 2, SEG><<<grid, kThreads, 0, s>>>(seg, pr, kIp0);
        k_sub2_norm<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src);
        k_scale_dots2<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src, 1);
        k_sub2_norm<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src);
        k_scale_dots2<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src, 1);
        k_sub2_norm<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src);
        k_scale_dots2<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src, 0);
        k_sub2_norm<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, src);
        k_mask<V, SEG><<<grid, kThreads, 0, s>>>(seg, src, v.p);
    }

    // one loop iteration (ground_locg.py:288-341)
    int iteration(int variant, cudaStream_t s) {
        V *src = v.r;
        if (jacobi) {
            k_jacobi<V, SEG><<<grid, kThreads, 0, s>>>(seg, diag, v.r, v.w);
            src = v.w;
        }
        project(src, s, variant);
        if (variant == RQ_LOBPCG_REFERENCE) {
            RQ_TRY(matvec(v.x, v.ax, s));
            RQ_TRY(matvec(v.y, v.ay, s));
        }
        RQ_TRY(matvec(v.p, v.ap, s));
        k_gram3<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p, v.ax, v.ay, v.ap);
        k_rr3<<<pgrid(), 128, 0, s>>>(states, P);
        if (variant == RQ_LOBPCG_FAST) {
            k_upd_stu<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p);
            k_stu_coef<<<pgrid(), 128, 0, s>>>(states, P);
        } else {
            k_upd_s<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.y, v.p);
            k_upd_tu<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p);
        }
        if (variant == RQ_LOBPCG_REFERENCE) {
            k_upd_xy<V, false, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p, nullptr, nullptr,
                                                              nullptr);
            RQ_TRY(matvec(v.x, v.ax, s));
        } else {
            k_upd_xy<V, true, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p, v.ax, v.ay, v.ap);
            // periodic / certifying refresh of the carried products
            RQ_TRY(matvec(v.x, v.ax, s, true));
            RQ_TRY(matvec(v.y, v.ay, s, true));
            k_refresh_mark<<<pgrid(), 128, 0, s>>>(states, P);
        }
        k_resid<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.ax, v.x, v.r, 0);
        k_check<<<pgrid(), 128, 0, s>>>(states, P, nactive);
        RQ_CUDA(cudaGetLastError());
        return RQ_OK;
    }

    // iterations 0 and 1 from v.x (unnormalised), ground_locg.py:264-286, 346; FAST also needs
    // A y for its carried products.  orth (restarts only): r is projected against x before it
    // becomes p.  r = A x - rho x carries a rounding component along x of order eps |A x|; from a
    // nearly converged x (|r| ~ 1e-8 |A x| in FP64) that makes <x, p> ~ 1e-7, and the two-term
    // Rayleigh-Ritz, which takes (x, p) as orthonormal, then moves x away from the eigenvector
    // (|r| 1.4e-8 -> 3e-6 in one step).  The reference's own start has |r| of order |A x|.
    int start(int variant, cudaStream_t s, bool orth = false) {
        Pairs<V, 1> nx{{v.x}, {v.x}};
        k_dots<V, 1, SEG><<<grid, kThreads, 0, s>>>(seg, nx, kMisc2);
        k_normalize<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.x, kMisc2);
        RQ_TRY(matvec(v.x, v.ax, s));
        Pairs<V, 1> rho{{v.x}, {v.ax}};
        k_dots<V, 1, SEG><<<grid, kThreads, 0, s>>>(seg, rho, kMisc);
        k_resid<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.ax, v.x, v.r, 1);
        int nslot = kRn;
        if (orth) {
            Pairs<V, 1> xr{{v.x}, {v.r}};
            k_dots<V, 1, SEG><<<grid, kThreads, 0, s>>>(seg, xr, kIp0);
            k_clear_slot<<<pgrid(), 128, 0, s>>>(states, P, kIp1);
            k_sub2_norm<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.x, v.r);  // r -= x <x, r>
            nslot = kVn;
        }
        // iteration 1: p = r / |r|
        k_normalize<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.r, v.p, nslot);
        RQ_TRY(matvec(v.x, v.ax, s));
        RQ_TRY(matvec(v.p, v.ap, s));
        k_gram2<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.p, v.ax, v.ap);
        k_rr2<<<pgrid(), 128, 0, s>>>(states, P);
        k_upd2_norms<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.p);
        k_upd2_xy<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.x, v.y, v.p);
        RQ_TRY(matvec(v.x, v.ax, s));
        if (variant == RQ_LOBPCG_FAST) RQ_TRY(matvec(v.y, v.ay, s));
        k_resid<V, SEG><<<grid, kThreads, 0, s>>>(seg, v.ax, v.x, v.r, 0);
        RQ_CUDA(cudaGetLastError());
        return RQ_OK;
    }
};

int read_active(const int *nactive, int &h, cudaStream_t s) {
    RQ_CUDA(cudaMemcpyAsync(&h, nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    return RQ_OK;
}

// Run iterations until no problem is active (or no more than stop_below).  With use_graph the
// chunk is captured once and relaunched; otherwise launched eagerly.  Callbacks run one iteration
// per chunk.
template <typename PH>
int run_loop(PH &ph, int variant, bool use_graph, int chunk, cudaStream_t s, int stop_below = 0) {
    int active = 0;
    auto enqueue_chunk = [&](cudaStream_t cs) -> int {
        for (int k = 0; k < chunk; ++k) RQ_TRY(ph.iteration(variant, cs));
        return RQ_OK;
    };
    if (!use_graph) {
        while (true) {
            RQ_TRY(enqueue_chunk(s));
            RQ_TRY(read_active(ph.nactive, active, s));
            if (active <= stop_below) break;
        }
        return RQ_OK;
    }
    cudaGraphExec_t exec = nullptr;
    auto capture = [&]() -> int {
        cudaGraph_t graph = nullptr;
        RQ_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_chunk(s);
        cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (rc != RQ_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        RQ_CUDA(e);
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        RQ_CUDA(e);
        return RQ_OK;
    };
    RQ_TRY(capture());
    int rc = RQ_OK;
    cudaError_t e = cudaSuccess;
    int last = ph.P;  // active problems when the block list was last rebuilt
    while (true) {
        e = cudaGraphLaunch(exec, s);
        if (e != cudaSuccess) break;
        rc = read_active(ph.nactive, active, s);
        if (rc != RQ_OK || active <= stop_below) break;
        if (ph.compact && active * 4 <= last) {
            // most problems have converged: launch blocks for the remaining ones only
            cudaGraphExecDestroy(exec);
            exec = nullptr;
            rc = ph.compact(ph.compact_ctx, active, &ph.grid, s);
            if (rc == RQ_OK) rc = capture();
            if (rc != RQ_OK) break;
            last = active;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (ph.compact && last != ph.P && rc == RQ_OK) rc = ph.compact(ph.compact_ctx, -1, &ph.grid, s);
    RQ_CUDA(e);
    return rc;
}

// ------------------------------------------------------------------------------------------
// Persistent LOBPCG: one cooperative launch runs a phase's iterations to convergence.  The passes
// are the same device bodies as the kernels above, separated by a grid barrier instead of a
// kernel boundary (a launch and its drain cost more than the work of a pass at D <= 2^20).
// ------------------------------------------------------------------------------------------
constexpr long long kBarrierCycles = 4000000000LL;  // ~2 s at 2 GHz: a barrier that waits longer aborts

// Grid barrier on a counter that only grows: each block adds 1 without waiting for the old value
// (the adds pipeline in L2 instead of queueing for their results) and waits until the counter
// reaches (barriers passed) x (blocks); `passed` is the block's own count, kept in shared
// memory.  Every wait is bounded; a block that gives up raises `abort`, which releases every
// other waiter at once.  Returns false after an abort.
__device__ bool group_sync(GridBar *b, unsigned int *passed, unsigned int nblocks) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned int target = (*passed + 1u) * nblocks;
        *passed += 1u;
        volatile unsigned int *count = &b->count;
        volatile int *abort = &b->abort;
        __threadfence();
        atomicAdd(&b->count, 1u);
        const long long t0 = clock64();
        while ((int)(*count - target) < 0) {
            if (*abort) {
                ok = 0;
                break;
            }
            if (clock64() - t0 > kBarrierCycles) {
                atomicExch(&b->abort, 1);
                ok = 0;
                break;
            }
        }
        __threadfence();
        if (*abort) ok = 0;
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// Barrier over the whole grid.
__device__ __forceinline__ bool grid_sync(GridBar *b, unsigned int *passed) {
    return group_sync(b, passed, gridDim.x);
}

// One problem inside the persistent kernel: every block holds its own copy of the solver state
// in shared memory.  A reduction writes the block's partial sums, crosses one grid barrier and
// then every block adds all partials itself in the same order, so the copies stay identical
// without a second barrier; scalar steps run on each block's thread 0.  Element i is always
// handled by the same thread, so passes that only touch a thread's own elements need no barrier.
struct SegPersist {
    State *st;      // this block's shared-memory copy
    int64_t D;
    float4 *part;   // [2][gridDim.x * kMaxReduce] partial sums, alternate reductions alternate
                    // halves (a block may write the next sums while another still reads these)
    GridBar *bar;
    int *flip;      // shared: which half the next reduction uses
    unsigned int *passed;  // shared: barriers this block has passed
    __device__ __forceinline__ State *state() const { return st; }
    __device__ __forceinline__ int64_t begin() const {
        return blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    }
    __device__ __forceinline__ int64_t end() const { return D; }
    __device__ __forceinline__ int64_t stride() const { return (int64_t)gridDim.x * blockDim.x; }
    template <int NV>
    __device__ void reduce(cdf (&v)[NV], int slot) const {
        __shared__ cdf red[kThreads / 32][NV];
        __shared__ cdf tot[NV];
        cdf w[NV];
        float4 *pb = part + (size_t)(*flip) * gridDim.x * kMaxReduce;
#pragma unroll
        for (int k = 0; k < NV; ++k) w[k] = v[k];
        block_sum_all<NV>(w, tot, red);
        if (threadIdx.x < NV) {
            pb[(size_t)blockIdx.x * kMaxReduce + threadIdx.x] = cdf_pack(tot[threadIdx.x]);
            __threadfence();
        }
        if (!grid_sync(bar, passed)) {
            if (threadIdx.x == 0) st->active = 0;  // aborted: every block stops
            __syncthreads();
            return;
        }
        partials_sum<NV>(pb, (int)gridDim.x, kMaxReduce, tot);
        if (threadIdx.x < NV) st->red[slot + threadIdx.x] = cdf_val(tot[threadIdx.x]);
        if (threadIdx.x == 0) *flip ^= 1;
        __syncthreads();
    }
};

// One problem of a batch inside the persistent batched kernel: blocks [b0, b0 + nb) of the grid
// (this block is number lb of them) own the problem's rows [r0, r1), reduce into the problem's
// own partial sums and cross the problem's own barrier; otherwise as SegPersist.
struct SegPersistB {
    State *st;
    int64_t r0, r1;
    int lb, nb;
    float4 *part;           // [2][nb * kMaxReduce]
    GridBar *bar;
    int *flip;
    unsigned int *passed;
    __device__ __forceinline__ State *state() const { return st; }
    __device__ __forceinline__ int64_t begin() const {
        return r0 + (int64_t)lb * blockDim.x + threadIdx.x;
    }
    __device__ __forceinline__ int64_t end() const { return r1; }
    __device__ __forceinline__ int64_t stride() const { return (int64_t)nb * blockDim.x; }
    template <int NV>
    __device__ void reduce(cdf (&v)[NV], int slot) const {
        __shared__ cdf red[kThreads / 32][NV];
        __shared__ cdf tot[NV];
        cdf w[NV];
        float4 *pb = part + (size_t)(*flip) * nb * kMaxReduce;
#pragma unroll
        for (int k = 0; k < NV; ++k) w[k] = v[k];
        block_sum_all<NV>(w, tot, red);
        if (threadIdx.x < NV) {
            pb[(size_t)lb * kMaxReduce + threadIdx.x] = cdf_pack(tot[threadIdx.x]);
            __threadfence();
        }
        if (!group_sync(bar, passed, (unsigned int)nb)) {
            if (threadIdx.x == 0) st->active = 0;
            __syncthreads();
            return;
        }
        partials_sum<NV>(pb, nb, kMaxReduce, tot);
        if (threadIdx.x < NV) st->red[slot + threadIdx.x] = cdf_val(tot[threadIdx.x]);
        if (threadIdx.x == 0) *flip ^= 1;
        __syncthreads();
    }
};

template <typename V>
struct PersistArgs {
    State *st;      // global state (read at start, written back by block 0 at the end)
    int64_t D;
    float4 *part;
    rq_operator_t op;
    Vecs<V> v;
    int variant;
    int jacobi;
    const double *diag;
    GridBar *bar;
};

// MVK 0: cached connectivity, 1: CSR with values of type V
template <typename V, int MVK>
__device__ __forceinline__ void persist_mv(const PersistArgs<V> &a, State *st, const V *in, V *out,
                                           const int *gate2) {
    if (MVK == 0)
        d_matvec_conn<V>(a.op, in, out, &st->active, gate2);
    else
        d_matvec_csr<V, V>(a.op, in, out, &st->active, gate2);
}

// The iterations of one phase inside a persistent kernel (ground_locg.py:288-341): the passes
// of Phase::iteration, separated by barriers of the segment instead of kernel boundaries.
// mv(in, out, gate2) forms a product over the segment's rows; sync() crosses the segment's
// barrier and returns false after an abort; the loop also ends at iteration stop_iter.  Element
// i is always handled by the same thread, so passes that only touch a thread's own elements need
// no barrier; barriers stand before the products (which gather rows of other blocks) and inside
// every reduction.
template <typename V, typename SEG, typename MVF, typename SYNC>
__device__ __forceinline__ void persist_loop(const SEG &seg, State *st, const Vecs<V> &v,
                                             int variant, int jacobi, const double *diag, MVF &mv,
                                             SYNC &sync, int stop_iter) {
    constexpr int kOnce = 1 << 30;  // step of the scalar loops: thread 0 only
    auto scalar_done = [&]() { __syncthreads(); };
    while (st->active && st->iter < stop_iter) {
        V *src = v.r;
        if (jacobi) {
            d_jacobi<V, SEG>(seg, diag, v.r, v.w);
            src = v.w;
        }
        // project_out((x, y), src) -> p
        if (variant == RQ_LOBPCG_FAST) {
            Pairs<V, 6> g{{v.x, v.y, v.x, v.x, v.y, src}, {src, src, v.x, v.y, v.y, src}};
            d_dots<V, 6, SEG>(seg, g, kG10);
            if (threadIdx.x == 0) d_proj_coef(st, 1, 0, kOnce);
            scalar_done();
            d_sub2_scale<V, SEG>(seg, v.x, v.y, src, v.p);
        } else {
            Pairs<V, 2> pr{{v.x, v.y}, {src, src}};
            d_dots<V, 2, SEG>(seg, pr, kIp0);
            d_sub2_norm<V, SEG>(seg, v.x, v.y, src);
            d_scale_dots2<V, SEG>(seg, v.x, v.y, src, 1);
            d_sub2_norm<V, SEG>(seg, v.x, v.y, src);
            d_scale_dots2<V, SEG>(seg, v.x, v.y, src, 1);
            d_sub2_norm<V, SEG>(seg, v.x, v.y, src);
            d_scale_dots2<V, SEG>(seg, v.x, v.y, src, 0);
            d_sub2_norm<V, SEG>(seg, v.x, v.y, src);
            d_mask<V, SEG>(seg, src, v.p);
        }
        if (!sync()) break;  // the products gather p (and x, y) from every block's rows
        if (variant == RQ_LOBPCG_REFERENCE) {
            mv(v.x, v.ax, nullptr);
            mv(v.y, v.ay, nullptr);
        }
        mv(v.p, v.ap, nullptr);
        d_gram3<V, SEG>(seg, v.x, v.y, v.p, v.ax, v.ay, v.ap);
        if (threadIdx.x == 0) d_rr3(st, 1, 0, kOnce);
        scalar_done();
        if (variant == RQ_LOBPCG_FAST) {
            d_upd_stu<V, SEG>(seg, v.x, v.y, v.p);
            if (threadIdx.x == 0) d_stu_coef(st, 1, 0, kOnce);
            scalar_done();
        } else {
            d_upd_s<V, SEG>(seg, v.y, v.p);
            d_upd_tu<V, SEG>(seg, v.x, v.y, v.p);
        }
        if (variant == RQ_LOBPCG_REFERENCE) {
            d_upd_xy<V, false, SEG>(seg, v.x, v.y, v.p, nullptr, nullptr, nullptr);
            if (!sync()) break;
            mv(v.x, v.ax, nullptr);
        } else {
            d_upd_xy<V, true, SEG>(seg, v.x, v.y, v.p, v.ax, v.ay, v.ap);
            if (st->want_refresh) {
                if (!sync()) break;
                mv(v.x, v.ax, &st->want_refresh);
                mv(v.y, v.ay, &st->want_refresh);
                if (threadIdx.x == 0) d_refresh_mark(st, 1, 0, kOnce);
                scalar_done();
            }
        }
        d_resid<V, SEG>(seg, v.ax, v.x, v.r, 0);
        if (threadIdx.x == 0) d_check(st, 1, nullptr, 0, kOnce);
        scalar_done();
    }
}

template <typename V, int MVK>
__global__ void __launch_bounds__(kThreads) k_persist(const PersistArgs<V> a) {
    __shared__ State sst;
    __shared__ int flip;
    __shared__ unsigned int passed;
    if (threadIdx.x == 0) {
        flip = 0;
        passed = 0u;
    }
    {
        const int n = (int)(sizeof(State) / sizeof(int));
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            reinterpret_cast<int *>(&sst)[k] = reinterpret_cast<const int *>(a.st)[k];
    }
    __syncthreads();
    State *st = &sst;
    const SegPersist seg{st, a.D, a.part, a.bar, &flip, &passed};
    auto sync = [&]() -> bool {
        if (grid_sync(a.bar, &passed)) return true;
        if (threadIdx.x == 0) st->active = 0;
        __syncthreads();
        return false;
    };
    auto mv = [&](const V *in, V *out, const int *gate2) { persist_mv<V, MVK>(a, st, in, out, gate2); };
    persist_loop<V, SegPersist>(seg, st, a.v, a.variant, a.jacobi, a.diag, mv, sync, INT_MAX);
    // the copies are identical; block 0 publishes its own
    if (blockIdx.x == 0) {
        const int n = (int)(sizeof(State) / sizeof(int));
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            reinterpret_cast<int *>(a.st)[k] = reinterpret_cast<const int *>(&sst)[k];
    }
}

// The batched cached-connectivity product over one problem's rows (the batch matvec's CONN form
// restricted to the segment): y[i] = diag0[i] x[i] + the row's cached (source, group) terms.
template <typename V>
__device__ __forceinline__ void d_batch_conn_seg(const rq_batch_t &B, const SegPersistB &seg,
                                                 const V *x, V *y, const int *gate2) {
    using R = typename VT<V>::R;
    if (!seg.st->active || (gate2 && *gate2 == 0)) return;
    constexpr uint64_t kMask = (1ULL << RQ_BATCH_STATE_BITS) - 1ULL;
    SEG_LOOP(i) {
        const uint64_t s = __ldg(B.keys + i) & kMask;
        CAcc<R> acc;
        const cx<R> xi = VT<V>::ld(x, i);
        const R dv = (R)B.diag0[i];
        acc.add({dv * xi.re, dv * xi.im});
        const int64_t e1 = B.rowptr[i + 1];
        for (int64_t e = B.rowptr[i]; e < e1; ++e)
            acc.add(cmul(group_diag<R>(B.terms, __ldg(B.grp + e), s), VT<V>::ld(x, __ldg(B.col + e))));
        VT<V>::st(y, i, acc.get());
    }
}

template <typename V>
struct PersistBatchArgs {
    State *states;          // [P], read at start, written back by each problem's first block
    rq_batch_t B;
    Vecs<V> v;
    int variant, jacobi;
    const double *diag;
    int iter_cap;           // iterations per problem in this launch
    const int32_t *bprob;   // [grid] problem of each block
    const int32_t *bfirst;  // [P] first block of each problem
    const int32_t *nblk;    // [P] blocks of each problem
    const int64_t *poff;    // [P] first float4 of each problem's partial sums
    float4 *part;
    GridBar *bars;          // [P]
};

// Many problems in one cooperative launch: each problem owns a group of blocks and runs
// persist_loop on its own rows with its own reductions and barrier (blocks of different problems
// never wait for each other), at most iter_cap iterations, after which the host re-plans the
// block groups over the problems still active.
template <typename V>
__global__ void __launch_bounds__(kThreads, 2) k_persist_batch(const PersistBatchArgs<V> a) {
    __shared__ State sst;
    __shared__ int flip;
    __shared__ unsigned int passed;
    const int q = a.bprob[blockIdx.x];
    if (threadIdx.x == 0) {
        flip = 0;
        passed = 0u;
    }
    {
        const int n = (int)(sizeof(State) / sizeof(int));
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            reinterpret_cast<int *>(&sst)[k] = reinterpret_cast<const int *>(a.states + q)[k];
    }
    __syncthreads();
    State *st = &sst;
    const int nb = a.nblk[q], lb = blockIdx.x - a.bfirst[q];
    const SegPersistB seg{st, a.B.prow[q], a.B.prow[q + 1], lb, nb, a.part + a.poff[q],
                          a.bars + q, &flip, &passed};
    auto sync = [&]() -> bool {
        if (group_sync(a.bars + q, &passed, (unsigned int)nb)) return true;
        if (threadIdx.x == 0) st->active = 0;
        __syncthreads();
        return false;
    };
    auto mv = [&](const V *in, V *out, const int *gate2) { d_batch_conn_seg<V>(a.B, seg, in, out, gate2); };
    const int stop = sst.iter + a.iter_cap;
    persist_loop<V, SegPersistB>(seg, st, a.v, a.variant, a.jacobi, a.diag, mv, sync, stop);
    if (lb == 0) {
        const int n = (int)(sizeof(State) / sizeof(int));
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            reinterpret_cast<int *>(a.states + q)[k] = reinterpret_cast<const int *>(&sst)[k];
    }
}

template <typename PH>
int run_persist(PH &ph, int variant, cudaStream_t s) {
    using V = typename std::remove_pointer<decltype(ph.v.x)>::type;
    const rq_operator_t &op = *ph.pop;
    const void *kern = op.mode == RQ_MODE_CONN ? (const void *)k_persist<V, 0> : (const void *)k_persist<V, 1>;
    int per = 0;
    RQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kThreads, 0));
    if (per < 1) return run_loop(ph, variant, true, kChunk, s);
    // as many blocks as the phase's kernels use, within the co-resident limit (the element-wise
    // FP64 work needs every SM; fewer, longer threads measured slower at D = 2^16)
    int grid = ph.grid;
    if (grid > per * sm_count()) grid = per * sm_count();
    if (grid > kMaxReduceBlocks / 2) grid = kMaxReduceBlocks / 2;  // two halves of partial sums
    // partial sums in the phase's reduction scratch (its counter slot stays unused)
    float4 *part = reinterpret_cast<float4 *>(static_cast<char *>(ph.seg.red) + 16);
    PersistArgs<V> a{ph.states, ph.seg.D, part, op, ph.v, variant, ph.jacobi ? 1 : 0, ph.diag,
                     ph.bar};
    RQ_CUDA(cudaMemsetAsync(ph.bar, 0, sizeof(GridBar), s));
    void *args[] = {&a};
    RQ_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kThreads), args, 0, s));
    GridBar h{};
    RQ_CUDA(cudaMemcpyAsync(&h, ph.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    if (h.abort) return fail(RQ_E_CUDA, "persistent LOBPCG: a grid barrier timed out");
    return RQ_OK;
}

// Device areas and the host copy of the row ranges of a persistent batched solve.
constexpr int kMaxPersistBlocks = 4096;
constexpr int kPersistIterCap = 256;         // iterations per launch before the blocks re-plan
constexpr int64_t kPersistRowsPerBlock = 1024;
struct BatchPersist {
    const rq_batch_t *b;
    std::vector<int64_t> prow;  // host copy
    int32_t *bprob, *bfirst, *nblk;
    int64_t *poff;
    GridBar *bars;
    float4 *part;
};

// A batched phase with persistent launches for its tail.  While more problems are active than a
// quarter of the co-resident blocks, CUDA-graph chunks run them (blocks of 2048 rows: every row of
// every problem gets a thread group, however many problems there are).  Then every launch gives
// each remaining problem a group of co-resident blocks (one block, plus a share of the rest in
// proportion to its rows, at most one per kPersistRowsPerBlock rows) and runs up to
// kPersistIterCap iterations; the host re-plans over the problems still active, so that the slow
// problems of the tail get the blocks of those that converged.
template <typename PH>
int run_persist_batch(PH &ph, int variant, cudaStream_t s) {
    using V = typename std::remove_pointer<decltype(ph.v.x)>::type;
    BatchPersist &bp = *ph.bp;
    const int P = ph.P;
    int per = 0;
    RQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_persist_batch<V>, kThreads, 0));
    int G = per * sm_count();
    if (G > kMaxPersistBlocks) G = kMaxPersistBlocks;
    std::vector<State> h(P);
    std::vector<int32_t> bprob, bfirst(P, 0), nblk(P, 0);
    std::vector<int64_t> poff(P, 0);
    std::vector<GridBar> bars(P);
    while (true) {
        RQ_CUDA(cudaMemcpyAsync(h.data(), ph.states, sizeof(State) * P, cudaMemcpyDeviceToHost, s));
        RQ_CUDA(cudaStreamSynchronize(s));
        int64_t rows = 0;
        int nact = 0;
        for (int q = 0; q < P; ++q)
            if (h[q].active) {
                rows += bp.prow[q + 1] - bp.prow[q];
                ++nact;
            }
        if (nact == 0) break;
        if (per < 1) return run_loop(ph, variant, true, kChunk, s);
        if (nact > G / 4) {  // many problems: graph chunks until a quarter of G remain
            RQ_CUDA(cudaMemcpyAsync(ph.nactive, &nact, sizeof(int), cudaMemcpyHostToDevice, s));
            RQ_CUDA(cudaStreamSynchronize(s));
            RQ_TRY(run_loop(ph, variant, true, kChunk, s, G / 4));
            continue;
        }
        const int extra = G - nact;
        bprob.clear();
        int64_t pos = 0;
        for (int q = 0; q < P; ++q) {
            nblk[q] = 0;
            bfirst[q] = (int32_t)bprob.size();
            poff[q] = pos;
            if (!h[q].active) continue;
            const int64_t r = bp.prow[q + 1] - bp.prow[q];
            const int64_t cap = std::max<int64_t>(1, (r + kPersistRowsPerBlock - 1) / kPersistRowsPerBlock);
            const int64_t n = 1 + (int64_t)((double)extra * (double)r / (double)rows);
            nblk[q] = (int32_t)std::min(n, cap);
            for (int k = 0; k < nblk[q]; ++k) bprob.push_back(q);
            pos += 2 * (int64_t)nblk[q] * kMaxReduce;
        }
        const int grid = (int)bprob.size();
        RQ_CUDA(cudaMemcpyAsync(bp.bprob, bprob.data(), sizeof(int32_t) * grid, cudaMemcpyHostToDevice, s));
        RQ_CUDA(cudaMemcpyAsync(bp.bfirst, bfirst.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, s));
        RQ_CUDA(cudaMemcpyAsync(bp.nblk, nblk.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, s));
        RQ_CUDA(cudaMemcpyAsync(bp.poff, poff.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, s));
        RQ_CUDA(cudaMemsetAsync(bp.bars, 0, sizeof(GridBar) * P, s));
        PersistBatchArgs<V> a{ph.states, *bp.b, ph.v, variant, ph.jacobi ? 1 : 0, ph.diag,
                              kPersistIterCap, bp.bprob, bp.bfirst, bp.nblk, bp.poff, bp.part,
                              bp.bars};
        void *args[] = {&a};
        RQ_CUDA(cudaLaunchCooperativeKernel((const void *)k_persist_batch<V>, dim3(grid),
                                            dim3(kThreads), args, 0, s));
        RQ_CUDA(cudaMemcpyAsync(bars.data(), bp.bars, sizeof(GridBar) * P, cudaMemcpyDeviceToHost, s));
        RQ_CUDA(cudaStreamSynchronize(s));  // (the host vectors above are read by the copies)
        for (int q = 0; q < P; ++q)
            if (bars[q].abort) return fail(RQ_E_CUDA, "persistent batched LOBPCG: a barrier timed out");
    }
    const int zero = 0;
    RQ_CUDA(cudaMemcpyAsync(ph.nactive, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    return RQ_OK;
}

// The iterations of one phase: a persistent kernel when the phase allows it, else CUDA-graph
// chunks (or eager launches).
template <typename PH>
int run_iterations(PH &ph, int variant, bool graph, int chunk, cudaStream_t s) {
    if constexpr (std::is_same<typename std::decay<decltype(ph.seg)>::type, SegOne>::value) {
        if (ph.pop && ph.bar) return run_persist(ph, variant, s);  // set only where allowed
    }
    if constexpr (std::is_same<typename std::decay<decltype(ph.seg)>::type, SegBatch>::value) {
        if (graph && ph.bp) return run_persist_batch(ph, variant, s);
    }
    return run_loop(ph, variant, graph, chunk, s);
}

// Per-problem state initialisation (tol_dim per problem), and the count of active problems.
int init_states(State *dev, int *nactive, int P, const rq_lobpcg_params_t &p, double tol,
                const std::vector<double> &tol_dim, bool lo, cudaStream_t s) {
    std::vector<State> h(P);
    for (int q = 0; q < P; ++q) {
        State &st = h[q];
        std::memset(&st, 0, sizeof(State));
        st.tol = tol;
        st.tol_dim = tol_dim[q];
        st.switch_rel = p.switch_rel > 0 ? p.switch_rel : 1e-5;
        st.target_rel = lo ? 0. : p.target_rel;
        st.best_r = INFINITY;
        st.maxiter = p.maxiter;
        st.active = 1;
        st.phase_lo = lo ? 1 : 0;
        st.refresh = p.refresh > 0 ? p.refresh : 32;
        st.variant = p.variant;
        st.guard = p.guard;
    }
    RQ_CUDA(cudaMemcpyAsync(dev, h.data(), sizeof(State) * P, cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(nactive, &P, sizeof(int), cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));  // host sources are stack objects
    return RQ_OK;
}

double eps_of(int32_t vt) {
    return (vt == RQ_F32 || vt == RQ_C64) ? 1.1920928955078125e-07 : 2.220446049250313e-16;
}

void fill_result(const State &h, int niter_lo, const rq_lobpcg_params_t &p, rq_lobpcg_result_t *res) {
    res->eigval = p.maxiter > 0 ? h.theta : 0.;  // the loop's initial theta (ground_locg.py:358)
    res->resnorm = h.resnorm;
    res->axnorm = h.axnorm;
    res->niter = h.iter + niter_lo;
    res->niter_lo = niter_lo;
    res->matvecs = 0;
    res->converged = h.converged;
    res->status = h.status ? h.status : (h.converged ? RQ_OK : RQ_E_MAXITER);
}

// run_iterations with a restart every `every` iterations (one problem, FAST variant; every <= 0:
// none): the phase stops at the restart point through its iteration limit, then the search
// direction y is dropped and the two-term step is taken again from x (the phase's start(), with
// r projected against x), with fresh products.  Long runs of the three-term step lose its
// conditioning; restarting every 100 iterations measured 290 -> 165 iterations (FP64, Hubbard
// D = 2^20).  Iterations keep counting across restarts, so maxiter is still the phase's total.
template <typename PH>
int run_iterations_restarting(PH &ph, int variant, bool graph, int chunk, cudaStream_t s, int every) {
    if (every <= 0 || ph.P != 1 || variant != RQ_LOBPCG_FAST) return run_iterations(ph, variant, graph, chunk, s);
    State h{};
    RQ_CUDA(cudaMemcpyAsync(&h, ph.states, sizeof(State), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    const int limit = h.maxiter;
    while (true) {
        const int stop = (int)std::min<int64_t>(limit, (int64_t)h.iter + every);
        RQ_CUDA(cudaMemcpyAsync(&ph.states->maxiter, &stop, sizeof(int), cudaMemcpyHostToDevice, s));
        RQ_TRY(run_iterations(ph, variant, graph, chunk, s));
        RQ_CUDA(cudaMemcpyAsync(&h, ph.states, sizeof(State), cudaMemcpyDeviceToHost, s));
        RQ_CUDA(cudaStreamSynchronize(s));  // `stop` is a stack object
        if (h.converged || h.status != 0 || h.iter >= limit) break;
        h.maxiter = limit;
        h.active = 1;
        h.since_refresh = 0;
        h.want_refresh = 0;
        h.certify = 0;
        const int one = 1;
        RQ_CUDA(cudaMemcpyAsync(ph.states, &h, sizeof(State), cudaMemcpyHostToDevice, s));
        RQ_CUDA(cudaMemcpyAsync(ph.nactive, &one, sizeof(int), cudaMemcpyHostToDevice, s));
        RQ_TRY(ph.start(variant, s, true));
        RQ_CUDA(cudaStreamSynchronize(s));  // h and `one` are stack objects
    }
    h.maxiter = limit;  // the state as a run without restarts would leave it
    RQ_CUDA(cudaMemcpyAsync(&ph.states->maxiter, &h.maxiter, sizeof(int), cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    return RQ_OK;
}

// Two-phase driver shared by the single-problem and the batched solves: an optional 32-bit phase,
// then the final value type.  `mk_lo` / `mk_hi` build the phases over their vectors.
template <typename PLO, typename PHI>
int run_phases(PLO &lo, PHI &hi, bool mixed, const rq_lobpcg_params_t &p, double tol,
               const std::vector<double> &tol_dim, int64_t D, const void *x0, size_t hi_bytes,
               int chunk, bool graph, cudaStream_t s, std::vector<int> &niter_lo) {
    using VLO = typename std::remove_pointer<decltype(lo.v.x)>::type;
    using VHI = typename std::remove_pointer<decltype(hi.v.x)>::type;
    const int P = hi.P;
    niter_lo.assign(P, 0);
    const int gconv = (int)std::min<int64_t>((D + kThreads - 1) / kThreads, (int64_t)sm_count() * 8);
    if (mixed) {
        RQ_TRY(init_states(lo.states, lo.nactive, P, p, eps_of(lo.vtype), tol_dim, true, s));
        k_convert<VHI, VLO><<<gconv, kThreads, 0, s>>>(D, static_cast<const VHI *>(x0), lo.v.x);
        RQ_TRY(lo.start(p.variant, s));
        if (p.maxiter > 0) RQ_TRY(run_iterations_restarting(lo, p.variant, graph, chunk, s, p.restart));
        std::vector<State> h(P);
        RQ_CUDA(cudaMemcpyAsync(h.data(), lo.states, sizeof(State) * P, cudaMemcpyDeviceToHost, s));
        RQ_CUDA(cudaStreamSynchronize(s));
        for (int q = 0; q < P; ++q) niter_lo[q] = h[q].iter;
        // restart in the final type from x alone: the 32-bit phase's search direction y is mostly
        // rounding noise once the residual nears the 32-bit floor, and a three-term step that
        // carries it on converges at the rate of steepest descent (thousands of iterations where
        // a restart from x takes a few hundred)
        k_convert<VLO, VHI><<<gconv, kThreads, 0, s>>>(D, lo.v.x, hi.v.x);
        RQ_TRY(init_states(hi.states, hi.nactive, P, p, tol, tol_dim, false, s));
        RQ_TRY(hi.start(p.variant, s));
    } else {
        RQ_TRY(init_states(hi.states, hi.nactive, P, p, tol, tol_dim, false, s));
        RQ_CUDA(cudaMemcpyAsync(hi.v.x, x0, hi_bytes, cudaMemcpyDeviceToDevice, s));
        RQ_TRY(hi.start(p.variant, s));
    }
    if (p.maxiter > 0) RQ_TRY(run_iterations_restarting(hi, p.variant, graph, chunk, s, p.restart));
    return RQ_OK;
}

template <typename VLO, typename VHI, typename MV>
int solve(const rq_operator_t &op, MV mv, bool callback, const rq_lobpcg_params_t &p, char *ws,
          const void *x0, void *xout, rq_lobpcg_result_t *res, cudaStream_t s) {
    const int64_t D = op.sub.D;
    const Layout L = layout(D, p);
    State *st = reinterpret_cast<State *>(ws + L.state);
    int *nactive = reinterpret_cast<int *>(ws + L.err + 8);
    void *red = ws + L.red;
    RQ_CUDA(cudaMemsetAsync(ws + L.err, 0, 64, s));
    RQ_CUDA(cudaMemsetAsync(red, 0, 16, s));
    const std::vector<double> tol_dim(1, p.tol_dim > 0 ? p.tol_dim : (double)D);
    const bool jac = p.jacobi != 0 && op.diag0 != nullptr;
    const int grid = grid_vec(D);
    const int32_t hi_type = p.vtype;
    const double tol = p.tol > 0 ? p.tol : eps_of(hi_type);
    const bool mixed = p.mixed && lo_type(hi_type) != hi_type;
    SegOne seg{st, D, red};
    Phase<VHI, SegOne, MV> hi{mv, hi_type, seg, grid, st, 1, nactive,
                              carve_vecs<VHI>(ws + L.vec_hi, L.hi_bytes), jac, op.diag0};
    Phase<VLO, SegOne, MV> lo{mv, lo_type(hi_type), seg, grid, st, 1, nactive,
                              carve_vecs<VLO>(ws + (mixed ? L.vec_lo : L.vec_hi), L.lo_bytes),
                              jac, op.diag0};
    std::vector<int> nlo;
    // use_graph 1: persistent kernel where the operator allows it, else graph chunks; 2: graph
    // chunks only; 3: persistent kernel where allowed, else eager launches (no graph); 0: eager
    const bool graph = (p.use_graph == 1 || p.use_graph == 2) && !callback;
    const bool persist = (p.use_graph == 1 || p.use_graph == 3) && !callback;
    // (the Jacobi preconditioner measured slower inside the persistent kernel: graphs then)
    if (persist && !jac && (op.mode == RQ_MODE_CONN || op.mode == RQ_MODE_CSR)) {
        // one persistent kernel per phase; CSR values must be of the phase's own type
        GridBar *bar = reinterpret_cast<GridBar *>(ws + L.err + 16);
        if (op.mode == RQ_MODE_CONN || op.val_vtype == hi_type) {
            hi.pop = &op;
            hi.bar = bar;
        }
        if (op.mode == RQ_MODE_CONN || op.val_vtype == lo.vtype) {
            lo.pop = &op;
            lo.bar = bar;
        }
    }
    RQ_TRY(run_phases(lo, hi, mixed, p, tol, tol_dim, D, x0, L.hi_bytes, callback ? 1 : kChunk,
                      graph, s, nlo));
    State h{};
    int mv_err = 0;
    RQ_CUDA(cudaMemcpyAsync(&h, st, sizeof(State), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaMemcpyAsync(&mv_err, ws + L.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaMemcpyAsync(xout, hi.v.x, L.hi_bytes, cudaMemcpyDeviceToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    if (mv_err) return fail(mv_err, "rq_lobpcg_solve: matvec reported an error");
    fill_result(h, nlo[0], p, res);
    return RQ_OK;
}

__global__ void k_eig3_abi(const double *m, double *out) {
    // m row-major complex [3][3]
    auto at = [&](int r, int c) { return make_double2(m[2 * (3 * r + c)], m[2 * (3 * r + c) + 1]); };
    double lam;
    double2 v[3];
    eig3(at(1, 0), at(2, 0), at(2, 1), at(0, 0), at(1, 1), at(2, 2), lam, v);
    out[0] = lam;
    out[1] = 0.;
    for (int k = 0; k < 3; ++k) {
        out[2 + 2 * k] = v[k].x;
        out[3 + 2 * k] = v[k].y;
    }
}

}  // namespace

}  // namespace rq

using namespace rq;

RQ_API int rq_lobpcg_workspace_size(int64_t D, const rq_lobpcg_params_t *prm, size_t *bytes) {
    if (!prm || !bytes || D < 1) return fail(RQ_E_ARG, "rq_lobpcg_workspace_size: bad arguments");
    if (vtype_size(prm->vtype) == 0) return fail(RQ_E_ARG, "rq_lobpcg_workspace_size: bad vtype");
    *bytes = layout(D, *prm).total;
    return RQ_OK;
}

namespace rq {
namespace {
int solve_entry(const rq_operator_t *op, rq_matvec_fn fn, void *ctx, const rq_lobpcg_params_t *prm,
                void *workspace, const void *x0, void *x_out, rq_lobpcg_result_t *res,
                void *stream) {
    if (!op || !prm || !workspace || !x0 || !x_out || !res)
        return fail(RQ_E_ARG, "rq_lobpcg_solve: null argument");
    if (prm->maxiter < 0) return fail(RQ_E_ARG, "rq_lobpcg_solve: maxiter < 0");
    if (prm->variant != RQ_LOBPCG_REFERENCE && prm->variant != RQ_LOBPCG_FAST)
        return fail(RQ_E_ARG, "rq_lobpcg_solve: unknown variant");
    if (prm->restart < 0) return fail(RQ_E_ARG, "rq_lobpcg_solve: restart < 0");
    const int32_t vt = prm->vtype;
    if (!fn && (vt == RQ_F32 || vt == RQ_F64) && !op->terms.is_real)
        return fail(RQ_E_ARG, "rq_lobpcg_solve: real vectors need real coefficients");
    if (op->sub.D < 1) return fail(RQ_E_ARG, "rq_lobpcg_solve: D must be >= 1");
    std::memset(res, 0, sizeof(*res));
    cudaStream_t user = as_stream(stream);
    // graphs cannot be captured on the legacy default stream: use a private stream ordered
    // after the caller's work
    cudaStream_t s = user;
    cudaStream_t priv = nullptr;
    const bool graph = (prm->use_graph == 1 || prm->use_graph == 2) && !fn;  // may capture a graph
    if (graph && user == nullptr) {
        RQ_CUDA(cudaStreamCreateWithFlags(&priv, cudaStreamNonBlocking));
        RQ_CUDA(cudaDeviceSynchronize());
        s = priv;
    }
    char *ws = static_cast<char *>(workspace);
    int rc;
    const Layout L = layout(op->sub.D, *prm);
    void *mvscratch = ws + L.err - kScratchErr;  // the matvec's error flag at ws + L.err
#define RQ_SOLVE(VLO, VHI)                                                                   \
    (fn ? solve<VLO, VHI>(*op, MvCallback{fn, ctx}, true, *prm, ws, x0, x_out, res, s)       \
        : solve<VLO, VHI>(*op, MvOne{op, mvscratch}, false, *prm, ws, x0, x_out, res, s))
    switch (vt) {
        case RQ_F32: rc = RQ_SOLVE(float, float); break;
        case RQ_F64: rc = RQ_SOLVE(float, double); break;
        case RQ_C64: rc = RQ_SOLVE(float2, float2); break;
        case RQ_C128: rc = RQ_SOLVE(float2, double2); break;
        default: rc = fail(RQ_E_ARG, "rq_lobpcg_solve: bad vtype");
    }
#undef RQ_SOLVE
    if (priv) {
        cudaStreamSynchronize(priv);
        cudaStreamDestroy(priv);
    }
    return rc;
}
}  // namespace
}  // namespace rq

RQ_API int rq_lobpcg_solve(const rq_operator_t *op, const rq_lobpcg_params_t *prm, void *workspace,
                           const void *x0, void *x_out, rq_lobpcg_result_t *res, void *stream) {
    return solve_entry(op, nullptr, nullptr, prm, workspace, x0, x_out, res, stream);
}

RQ_API int rq_lobpcg_solve_cb(int64_t D, rq_matvec_fn fn, void *ctx, const rq_lobpcg_params_t *prm,
                              void *workspace, const void *x0, void *x_out, rq_lobpcg_result_t *res,
                              void *stream) {
    if (!fn) return fail(RQ_E_ARG, "rq_lobpcg_solve_cb: null callback");
    if (prm && prm->variant != RQ_LOBPCG_REFERENCE)
        return fail(RQ_E_ARG, "rq_lobpcg_solve_cb: callbacks run the REFERENCE variant");
    rq_operator_t op = {};
    op.sub.D = D;
    op.terms.diag_group = -1;
    op.terms.is_real = 1;
    return solve_entry(&op, fn, ctx, prm, workspace, x0, x_out, res, stream);
}

RQ_API int rq_eigenpair_3x3(const double *mat, double *out, void *stream) {
    if (!mat || !out) return fail(RQ_E_ARG, "rq_eigenpair_3x3: null argument");
    k_eig3_abi<<<1, 1, 0, as_stream(stream)>>>(mat, out);
    RQ_CUDA(cudaGetLastError());
    return RQ_OK;
}

namespace rq {

// ------------------------------------------------------------------------------------------
// Allocation-free solve
// ------------------------------------------------------------------------------------------
// For callers that must not allocate device memory themselves -- code running inside a
// framework that owns the allocator (a custom-call handler gets only its operand and result
// buffers; the framework's pool holds the rest of the memory) or a service whose device memory is
// reserved up front (a later cudaMalloc could fail or fragment the reserve).  The solver's
// workspace (reduction partials and counters, the matvec's error record, the iteration vectors)
// lives in this file-scope device array instead of caller memory.  Every GPU that loads the
// library holds it until the process exits.
namespace {

constexpr size_t kNoallocBytes = size_t(8) << 20;  // 8 MiB
static __device__ __align__(256) unsigned char g_noalloc_ws[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_ws on the current device.  In host code the symbol is only a
// host-side stand-in, so the address is looked up once per device (with that device current)
// and cached.
int noalloc_workspace(void **out) {
    int dev = 0;
    RQ_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(RQ_E_RANGE, "rq_lobpcg_solve_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        RQ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_ws));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return RQ_OK;
}

}  // namespace
}  // namespace rq

RQ_API int rq_lobpcg_solve_noalloc(const rq_operator_t *op, const rq_lobpcg_params_t *prm,
                                   const void *x0, void *x_out, rq_lobpcg_result_t *res,
                                   void *stream) {
    if (!op || !prm || !x0 || !x_out || !res)
        return fail(RQ_E_ARG, "rq_lobpcg_solve_noalloc: null argument");
    if (op->sub.D < 1) return fail(RQ_E_ARG, "rq_lobpcg_solve_noalloc: D must be >= 1");
    if (vtype_size(prm->vtype) == 0) return fail(RQ_E_ARG, "rq_lobpcg_solve_noalloc: bad vtype");
    const size_t need = layout(op->sub.D, *prm).total;
    if (need > kNoallocBytes)
        return fail(RQ_E_RANGE,
                    "rq_lobpcg_solve_noalloc: D = " + std::to_string(op->sub.D) + " needs " +
                        std::to_string(need) + " bytes of workspace; the static workspace holds " +
                        std::to_string(kNoallocBytes) + " bytes (use rq_lobpcg_solve)");
    void *ws = nullptr;
    RQ_TRY(noalloc_workspace(&ws));
    // No CUDA graph of its own: instantiating one may allocate device memory.  Cached-connectivity
    // and CSR operators run each precision phase as the persistent cooperative kernel (a launch
    // that allocates nothing), others launch every pass eagerly.  The workspace carries the last
    // call's contents; solve() clears the reduction counter, the grid barrier and the error record
    // it relies on.
    rq_lobpcg_params_t p = *prm;
    p.use_graph = 3;
    return solve_entry(op, nullptr, nullptr, &p, ws, x0, x_out, res, stream);
}

// ------------------------------------------------------------------------------------------
// Batched solve: every problem's rows in one vector, chunked segments, per-problem state
// ------------------------------------------------------------------------------------------
namespace rq {

int batch_matvec_dispatch(const rq_batch_t &B, int32_t vt, const void *x, void *y, void *scratch,
                          cudaStream_t st, const int *gate, int64_t gstride, const int *gate2);

namespace {

constexpr int64_t kBatchChunk = 2048;  // rows per block of the batched passes

struct MvBatch {
    const rq_batch_t *b;
    void *scratch;
    int operator()(int32_t vt, const void *in, void *out, cudaStream_t s, State *states,
                   bool refresh) const {
        return batch_matvec_dispatch(*b, vt, in, out, scratch, s, &states[0].active,
                                     (int64_t)sizeof(State),
                                     refresh ? &states[0].want_refresh : nullptr);
    }
};

struct BatchPlan {
    std::vector<int64_t> prow;
    std::vector<int32_t> cprob, cofs;
    std::vector<int64_t> crow, cend;
    size_t states, err, part, counter, tcprob, tcrow, tcend, tcofs, vec_hi, vec_lo, total;
    size_t pb_prob, pb_first, pb_nblk, pb_poff, pb_bars, pb_part;  // persistent launches
    size_t hi_bytes, lo_bytes;
};

int plan_batch(const rq_batch_t &b, const rq_lobpcg_params_t &p, BatchPlan &pl) {
    const int P = b.P;
    pl.prow.resize(P + 1);
    RQ_CUDA(cudaMemcpy(pl.prow.data(), b.prow, sizeof(int64_t) * (P + 1), cudaMemcpyDeviceToHost));
    if (pl.prow[0] != 0 || pl.prow[P] != b.D) return fail(RQ_E_ARG, "rq_batch: prow must span [0, D]");
    pl.cofs.assign(1, 0);
    for (int q = 0; q < P; ++q) {
        const int64_t a = pl.prow[q], e = pl.prow[q + 1];
        if (e <= a) return fail(RQ_E_ARG, "rq_batch: every problem needs at least one row");
        for (int64_t r = a; r < e; r += kBatchChunk) {
            pl.cprob.push_back(q);
            pl.crow.push_back(r);
            pl.cend.push_back(std::min(r + kBatchChunk, e));
        }
        pl.cofs.push_back((int32_t)pl.cprob.size());
    }
    pl.crow.push_back(b.D);
    const size_t nch = pl.cprob.size();
    size_t off = 0;
    auto take = [&](size_t n) {
        size_t o = off;
        off += (n + 255) & ~size_t(255);
        return o;
    };
    pl.states = take(sizeof(State) * P);
    pl.err = take(16);
    pl.part = take(sizeof(double2) * kMaxReduce * nch);
    pl.counter = take(sizeof(unsigned int) * P);
    pl.tcprob = take(sizeof(int32_t) * nch);
    pl.tcrow = take(sizeof(int64_t) * (nch + 1));
    pl.tcend = take(sizeof(int64_t) * nch);
    pl.tcofs = take(sizeof(int32_t) * (P + 1));
    pl.pb_prob = take(sizeof(int32_t) * kMaxPersistBlocks);
    pl.pb_first = take(sizeof(int32_t) * P);
    pl.pb_nblk = take(sizeof(int32_t) * P);
    pl.pb_poff = take(sizeof(int64_t) * P);
    pl.pb_bars = take(sizeof(GridBar) * P);
    pl.pb_part = take(sizeof(float4) * 2 * kMaxPersistBlocks * kMaxReduce);
    pl.hi_bytes = (size_t)b.D * vtype_size(p.vtype);
    pl.lo_bytes = (size_t)b.D * vtype_size(lo_type(p.vtype));
    pl.vec_hi = take(8 * ((pl.hi_bytes + 255) & ~size_t(255)));
    pl.vec_lo = p.mixed ? take(8 * ((pl.lo_bytes + 255) & ~size_t(255))) : 0;
    pl.total = off;
    return RQ_OK;
}

// Block lists of a batched solve: the full one, or the chunks of the problems still active.
struct BatchBlocks {
    const BatchPlan *pl;
    int P;
    State *states;
    int32_t *cprob;
    int64_t *crow, *cend;
    int32_t *cofs;
};

int batch_compact(void *vctx, int active, int *grid, cudaStream_t s) {
    BatchBlocks &c = *static_cast<BatchBlocks *>(vctx);
    const BatchPlan &pl = *c.pl;
    std::vector<int32_t> cprob, cofs(1, 0);
    std::vector<int64_t> crow, cend;
    if (active < 0) {  // restore
        cprob = pl.cprob;
        crow.assign(pl.crow.begin(), pl.crow.end() - 1);
        cend = pl.cend;
        cofs = pl.cofs;
    } else {
        std::vector<State> h(c.P);
        RQ_CUDA(cudaMemcpyAsync(h.data(), c.states, sizeof(State) * c.P, cudaMemcpyDeviceToHost, s));
        RQ_CUDA(cudaStreamSynchronize(s));
        for (int q = 0; q < c.P; ++q) {
            if (h[q].active)
                for (int k = pl.cofs[q]; k < pl.cofs[q + 1]; ++k) {
                    cprob.push_back(pl.cprob[k]);
                    crow.push_back(pl.crow[k]);
                    cend.push_back(pl.cend[k]);
                }
            cofs.push_back((int32_t)cprob.size());
        }
        if (cprob.empty()) return RQ_OK;  // nothing left: keep the list (every block returns)
    }
    const size_t n = cprob.size();
    RQ_CUDA(cudaMemcpyAsync(c.cprob, cprob.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(c.crow, crow.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(c.cend, cend.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(c.cofs, cofs.data(), sizeof(int32_t) * cofs.size(), cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));  // host vectors are temporaries
    *grid = (int)n;
    return RQ_OK;
}

template <typename VLO, typename VHI>
int solve_batch(const rq_batch_t &b, const rq_lobpcg_params_t &p, const BatchPlan &pl, char *ws,
                const void *x0, void *xout, rq_lobpcg_result_t *res, cudaStream_t s) {
    const int P = b.P;
    State *states = reinterpret_cast<State *>(ws + pl.states);
    int *nactive = reinterpret_cast<int *>(ws + pl.err + 8);
    unsigned int *counter = reinterpret_cast<unsigned int *>(ws + pl.counter);
    int32_t *cprob = reinterpret_cast<int32_t *>(ws + pl.tcprob);
    int64_t *crow = reinterpret_cast<int64_t *>(ws + pl.tcrow);
    int64_t *cend = reinterpret_cast<int64_t *>(ws + pl.tcend);
    int32_t *cofs = reinterpret_cast<int32_t *>(ws + pl.tcofs);
    RQ_CUDA(cudaMemsetAsync(ws + pl.err, 0, 16, s));
    RQ_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int) * P, s));
    RQ_CUDA(cudaMemcpyAsync(cprob, pl.cprob.data(), sizeof(int32_t) * pl.cprob.size(),
                            cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(crow, pl.crow.data(), sizeof(int64_t) * pl.crow.size(),
                            cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(cofs, pl.cofs.data(), sizeof(int32_t) * pl.cofs.size(),
                            cudaMemcpyHostToDevice, s));
    RQ_CUDA(cudaMemcpyAsync(cend, pl.cend.data(), sizeof(int64_t) * pl.cend.size(),
                            cudaMemcpyHostToDevice, s));
    std::vector<double> tol_dim(P);
    for (int q = 0; q < P; ++q) {
        const int64_t rows = pl.prow[q + 1] - pl.prow[q];
        if (b.states_size && b.states_size[q] < rows)
            return fail(RQ_E_ARG, "rq_batch_solve: states_size below a problem's row count");
        tol_dim[q] = (double)(b.states_size ? b.states_size[q] : rows);
    }
    const int32_t hi_type = p.vtype;
    const double tol = p.tol > 0 ? p.tol : eps_of(hi_type);
    const bool mixed = p.mixed && lo_type(hi_type) != hi_type;
    const int grid = (int)pl.cprob.size();
    SegBatch seg{states, cprob, crow, cend, cofs, reinterpret_cast<double2 *>(ws + pl.part), counter};
    void *mvscratch = ws + pl.err - kScratchErr;
    const bool jac = p.jacobi != 0;
    Phase<VHI, SegBatch, MvBatch> hi{MvBatch{&b, mvscratch}, hi_type, seg, grid, states, P, nactive,
                                     carve_vecs<VHI>(ws + pl.vec_hi, pl.hi_bytes), jac, b.diag0};
    Phase<VLO, SegBatch, MvBatch> lo{MvBatch{&b, mvscratch}, lo_type(hi_type), seg, grid, states, P,
                                     nactive,
                                     carve_vecs<VLO>(ws + (mixed ? pl.vec_lo : pl.vec_hi), pl.lo_bytes),
                                     jac, b.diag0};
    BatchBlocks blocks{&pl, P, states, cprob, crow, cend, cofs};
    hi.compact = lo.compact = batch_compact;
    hi.compact_ctx = lo.compact_ctx = &blocks;
    // cached connectivity: each phase as persistent launches (use_graph 2 keeps the graph chunks;
    // the Jacobi pass stays on the graph path, as for one problem)
    BatchPersist bp{&b, pl.prow,
                    reinterpret_cast<int32_t *>(ws + pl.pb_prob),
                    reinterpret_cast<int32_t *>(ws + pl.pb_first),
                    reinterpret_cast<int32_t *>(ws + pl.pb_nblk),
                    reinterpret_cast<int64_t *>(ws + pl.pb_poff),
                    reinterpret_cast<GridBar *>(ws + pl.pb_bars),
                    reinterpret_cast<float4 *>(ws + pl.pb_part)};
    if (p.use_graph == 1 && b.mode == RQ_MODE_CONN && !jac) hi.bp = lo.bp = &bp;
    std::vector<int> nlo;
    RQ_TRY(run_phases(lo, hi, mixed, p, tol, tol_dim, b.D, x0, pl.hi_bytes, kChunk,
                      p.use_graph != 0, s, nlo));
    std::vector<State> h(P);
    int mv_err = 0;
    RQ_CUDA(cudaMemcpyAsync(h.data(), states, sizeof(State) * P, cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaMemcpyAsync(&mv_err, ws + pl.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RQ_CUDA(cudaMemcpyAsync(xout, hi.v.x, pl.hi_bytes, cudaMemcpyDeviceToDevice, s));
    RQ_CUDA(cudaStreamSynchronize(s));
    if (mv_err) return fail(mv_err, "rq_batch_solve: matvec reported an error");
    for (int q = 0; q < P; ++q) fill_result(h[q], nlo[q], p, res + q);
    return RQ_OK;
}

}  // namespace
}  // namespace rq

RQ_API int rq_batch_workspace_size(const rq_batch_t *b, const rq_lobpcg_params_t *prm,
                                   size_t *bytes) {
    if (!b || !prm || !bytes || !b->prow || b->P < 1)
        return fail(RQ_E_ARG, "rq_batch_workspace_size: bad arguments");
    if (vtype_size(prm->vtype) == 0) return fail(RQ_E_ARG, "rq_batch_workspace_size: bad vtype");
    BatchPlan pl;
    RQ_TRY(plan_batch(*b, *prm, pl));
    *bytes = pl.total;
    return RQ_OK;
}

RQ_API int rq_batch_solve(const rq_batch_t *b, const rq_lobpcg_params_t *prm, void *workspace,
                          const void *x0, void *x_out, rq_lobpcg_result_t *res, void *stream) {
    if (!b || !prm || !workspace || !x0 || !x_out || !res)
        return fail(RQ_E_ARG, "rq_batch_solve: null argument");
    if (prm->maxiter < 0 || (prm->variant != RQ_LOBPCG_REFERENCE && prm->variant != RQ_LOBPCG_FAST))
        return fail(RQ_E_ARG, "rq_batch_solve: bad maxiter or variant");
    if (prm->restart < 0) return fail(RQ_E_ARG, "rq_batch_solve: restart < 0");
    const int32_t vt = prm->vtype;
    if ((vt == RQ_F32 || vt == RQ_F64) && !b->terms.is_real)
        return fail(RQ_E_ARG, "rq_batch_solve: real vectors need real coefficients");
    BatchPlan pl;
    RQ_TRY(plan_batch(*b, *prm, pl));
    std::memset(res, 0, sizeof(rq_lobpcg_result_t) * b->P);
    cudaStream_t user = as_stream(stream);
    cudaStream_t s = user, priv = nullptr;
    if (prm->use_graph && user == nullptr) {
        RQ_CUDA(cudaStreamCreateWithFlags(&priv, cudaStreamNonBlocking));
        RQ_CUDA(cudaDeviceSynchronize());
        s = priv;
    }
    char *ws = static_cast<char *>(workspace);
    int rc;
    switch (vt) {
        case RQ_F32: rc = solve_batch<float, float>(*b, *prm, pl, ws, x0, x_out, res, s); break;
        case RQ_F64: rc = solve_batch<float, double>(*b, *prm, pl, ws, x0, x_out, res, s); break;
        case RQ_C64: rc = solve_batch<float2, float2>(*b, *prm, pl, ws, x0, x_out, res, s); break;
        case RQ_C128: rc = solve_batch<float2, double2>(*b, *prm, pl, ws, x0, x_out, res, s); break;
        default: rc = fail(RQ_E_ARG, "rq_batch_solve: bad vtype");
    }
    if (priv) {
        cudaStreamSynchronize(priv);
        cudaStreamDestroy(priv);
    }
    return rc;
}
