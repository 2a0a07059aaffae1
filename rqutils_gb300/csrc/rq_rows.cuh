// Row products shared by the matvec launches and the persistent LOBPCG kernel: the diagonal of
// one X group on a row, and the cached-connectivity (CONN) and cached-element (CSR) row sums.
// The vectors are plain pointers (no __restrict__): inside the persistent kernel they are
// written by other blocks between grid barriers, so they must not be read through the
// non-coherent path.
#pragma once

#include "rq_common.cuh"

namespace rq {
namespace {

// sum_k c_k (-1)^popcount(s & z_k) over group g, stopping at the first zero coefficient
template <typename R>
__device__ __forceinline__ cx<R> group_diag(const rq_terms_t &T, int g, uint64_t s) {
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

// y[i] = diag0[i] x[i] + sum over the row's cached (source, group) pairs; gated like the kernels
template <typename V>
__device__ __forceinline__ void d_matvec_conn(const rq_operator_t &op, const V *x, V *y,
                                              const int *gate, const int *gate2) {
    using R = typename VT<V>::R;
    if (gate && (*gate == 0 || (gate2 && *gate2 == 0))) return;
    const rq_terms_t &T = op.terms;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.sub.D;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t s = __ldg(op.sub.states + i);
        CAcc<R> acc;
        const cx<R> xi = VT<V>::ld(x, i);
        if (op.diag0) {
            const R dv = (R)op.diag0[i];
            acc.add({dv * xi.re, dv * xi.im});
        } else if (T.diag_group >= 0) {
            acc.add(cmul(group_diag<R>(T, T.diag_group, s), xi));
        }
        const int64_t e1 = op.rowptr[i + 1];
        for (int64_t e = op.rowptr[i]; e < e1; ++e)
            acc.add(cmul(group_diag<R>(T, __ldg(op.grp + e), s), VT<V>::ld(x, __ldg(op.col + e))));
        VT<V>::st(y, i, acc.get());
    }
}

// y[i] = diag0[i] x[i] + sum over the row's cached elements (value type VV)
template <typename V, typename VV>
__device__ __forceinline__ void d_matvec_csr(const rq_operator_t &op, const V *x, V *y,
                                             const int *gate, const int *gate2) {
    using R = typename VT<V>::R;
    if (gate && (*gate == 0 || (gate2 && *gate2 == 0))) return;
    const VV *val = reinterpret_cast<const VV *>(op.val);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < op.sub.D;
         i += (int64_t)gridDim.x * blockDim.x) {
        CAcc<R> acc;
        if (op.diag0) {
            const R dv = (R)op.diag0[i];
            const cx<R> xi = VT<V>::ld(x, i);
            acc.add({dv * xi.re, dv * xi.im});
        }
        const int64_t e1 = op.rowptr[i + 1];
        for (int64_t e = op.rowptr[i]; e < e1; ++e) {
            const auto v = VT<VV>::ld(val, e);
            acc.add(cmul(cx<R>{(R)v.re, (R)v.im}, VT<V>::ld(x, __ldg(op.col + e))));
        }
        VT<V>::st(y, i, acc.get());
    }
}

}  // namespace
}  // namespace rq
