"""Oracle restatement of the SQD path of ``rqutils/sqd.py`` on uint64 bitstrings.

Test infrastructure only (see ``oracle/__init__.py``).  Every function names the reference lines
it restates.  Bit convention: bit ``q`` of a state is qubit ``q``; column 0 of a 0/1 row is qubit
``n-1`` (``sqd.py:237``), so the numeric order of the integers is the reference's sort order.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .paulis import from_paulisum, OracleTerms
from .ground_locg import ground_locg

_ONE = np.uint64(1)


def pack_states(states01):
    """(D, n) 0/1 rows -> uint64, column 0 the most significant qubit (sqd.py:237)."""
    states01 = np.asarray(states01).astype(np.uint64)
    n = states01.shape[1]
    weights = _ONE << np.arange(n - 1, -1, -1, dtype=np.uint64)
    return np.bitwise_or.reduce(states01 * weights, axis=1) if n else np.zeros(len(states01),
                                                                              np.uint64)


def unpack_states(states, n):
    """uint64 -> (D, n) uint8 rows, column 0 = qubit n-1 (sqd.py:246)."""
    states = np.asarray(states, dtype=np.uint64)
    shifts = np.arange(n - 1, -1, -1, dtype=np.uint64)
    return ((states[:, None] >> shifts[None, :]) & _ONE).astype(np.uint8)


def uniquify(states):
    """Sorted distinct states (uniquify_states, sqd.py:414-445, without the 0xFF fill rows)."""
    return np.unique(np.asarray(states, dtype=np.uint64))


def popparity(a):
    """popcount(a) & 1 for a uint64 array."""
    return (np.bitwise_count(a) & np.uint8(1)).astype(np.int64)


def xsource_sortmerge(states, xmask):
    """get_xsource, sqd.py:448-503: stable sort of [S; S^x] with an iota; equal neighbours pair row
    i of S with the source m where S[m] = S[i]^x; rows with no equal neighbour get -1.  The result
    is put back in row order by locating S's entries in the sorted list (sqd.py:493-500)."""
    S = np.asarray(states, dtype=np.uint64)
    N = S.shape[0]
    joined = np.concatenate([S, S ^ np.uint64(xmask)])
    order = np.argsort(joined, kind='stable')
    T = joined[order]
    src = np.where(T[:-1] == T[1:], order[1:] - N, -1)
    pos_s = np.nonzero(order < N)[0]
    out = np.full(N, -1, dtype=np.int64)
    inside = pos_s < 2 * N - 1
    out[inside] = src[pos_s[inside]]
    return out.astype(np.int32)


def xsource_search(states, xmask):
    """Same table as xsource_sortmerge via binary search (the lookup the GPU kernels perform)."""
    S = np.asarray(states, dtype=np.uint64)
    t = S ^ np.uint64(xmask)
    pos = np.searchsorted(S, t)
    posc = np.minimum(pos, len(S) - 1)
    hit = (pos < len(S)) & (S[posc] == t)
    return np.where(hit, pos, -1).astype(np.int32)


def diagonal(states, zrow, crow):
    """get_diagonal, sqd.py:554-575: sum_k c_k (1 - 2*parity(s & z_k)), stopping at the first
    coefficient equal to zero (padding, or a consolidated term that cancelled exactly)."""
    S = np.asarray(states, dtype=np.uint64)
    out = np.zeros(S.shape[0], dtype=np.asarray(crow).dtype)
    for zk, ck in zip(zrow, crow):
        if ck == 0:
            break
        out = out + ck * (1. - 2. * popparity(S & np.uint64(zk)))
    return out


def xsources_all(states, terms: OracleTerms):
    """The cached (J, D) int32 table, sqd.py:318-326."""
    return np.stack([xsource_sortmerge(states, xv) for xv in terms.x])


def gather_fill(vec, src):
    """vec[src] with 0 where src == -1 (apply_xgrp, sqd.py:585-587)."""
    return np.where(src >= 0, vec[np.maximum(src, 0)], 0)


def matvec_xcached(vec, xsources, terms: OracleTerms, states):
    """apply_h_x_cached, sqd.py:640-654: out = sum_j diag_j * vec[xsource_j] in group order."""
    out = np.zeros_like(vec)
    for j in range(len(terms.x)):
        out = out + gather_fill(vec, xsources[j]) * diagonal(states, terms.z[j], terms.c[j])
    return out


def _group_cuts(terms: OracleTerms):
    """Number of leading nonzero coefficients of each group: get_diagonal's loop ends at the first
    zero coefficient (sqd.py:561-564)."""
    c = np.asarray(terms.c)
    zero = c == 0
    first = np.where(zero.any(axis=1), zero.argmax(axis=1), c.shape[1])
    return first.astype(np.int64)


def rows_matvec(vec, terms: OracleTerms, states, rows, chunk=64, halves=None):
    """apply_h_x_cached (sqd.py:640-654) evaluated on selected rows only, for subspaces too large
    for the (J, D) table.  For row i and X group j the source is the position of S[i] ^ x_j in the
    sorted states (searchsorted: the same table as the sort-merge of get_xsource, sqd.py:448-503,
    which the fixtures check) or absent; the value is sum_j diag_j(S[i]) vec[source], the groups
    added in ascending order, each diagonal over the group's terms up to its first zero
    coefficient (sqd.py:554-575).

    ``halves`` = (A, B): optional qubit masks; a target whose (popcount(t & A), popcount(t & B))
    pair occurs for no state cannot be a state, so it is skipped before the search (an exact
    shortcut).  Returns (y[rows], hits) with hits a list, per row, of (group, source) pairs in
    ascending group order over the groups with x != 0."""
    S = np.asarray(states, dtype=np.uint64)
    rows = np.asarray(rows, dtype=np.int64)
    X = np.asarray(terms.x, dtype=np.uint64)
    Z = np.asarray(terms.z, dtype=np.uint64)
    C = np.asarray(terms.c)
    cut = _group_cuts(terms)
    nz = np.nonzero(X != 0)[0]
    dg = [int(j) for j in np.nonzero(X == 0)[0]]
    pairs = None
    if halves is not None:
        A, B = (np.uint64(h) for h in halves)
        pa, pb = np.bitwise_count(S & A).astype(np.int64), np.bitwise_count(S & B).astype(np.int64)
        pairs = np.unique(pa * 65 + pb)
    ydt = np.result_type(vec.dtype, C.dtype)
    y = np.zeros(len(rows), dtype=ydt)
    hits = []

    def diags(s, groups):
        if len(groups) == 0:
            return np.zeros(0, dtype=C.dtype)
        kc = int(cut[groups].max())
        zz, cc = Z[groups, :kc], C[groups, :kc]
        live = np.arange(kc)[None, :] < cut[groups][:, None]
        sign = 1. - 2. * (np.bitwise_count(zz & s) & np.uint8(1))
        return np.sum(np.where(live, cc * sign, 0), axis=1)

    for a in range(0, len(rows), chunk):
        rr = rows[a:a + chunk]
        t = S[rr][:, None] ^ X[None, nz]                   # (rows, groups with x != 0)
        if pairs is not None:
            key = (np.bitwise_count(t & A).astype(np.int64) * 65 +
                   np.bitwise_count(t & B).astype(np.int64))
            ri, gi = np.nonzero(np.isin(key, pairs))
        else:
            ri, gi = np.nonzero(np.ones(t.shape, dtype=bool))
        tt = t[ri, gi]
        pos = np.searchsorted(S, tt)
        posc = np.minimum(pos, len(S) - 1)
        found = (pos < len(S)) & (S[posc] == tt)
        ri, gi, src = ri[found], nz[gi[found]], pos[found]
        for k, i in enumerate(rr):
            sel = ri == k
            g_k, m_k = gi[sel], src[sel]
            order = np.argsort(g_k, kind='stable')
            g_k, m_k = g_k[order], m_k[order]
            hits.append(list(zip(g_k.tolist(), m_k.tolist())))
            s = S[i]
            groups = np.array(dg + g_k.tolist(), dtype=np.int64)
            srcs = np.array([int(i)] * len(dg) + m_k.tolist(), dtype=np.int64)
            d = diags(s, groups)
            order = np.argsort(groups, kind='stable')
            acc = ydt.type(0)
            for val in (d * vec[srcs])[order]:
                acc = acc + val
            y[a + k] = acc
    return y, hits


def matvec_nocache(vec, terms: OracleTerms, states, threads=1):
    """apply_h, sqd.py:590-605: the X sources are recomputed (sort-merge) inside every matvec.

    With ``threads > 1`` the groups are split over a thread pool (NumPy releases the GIL inside
    its sorts and ufuncs) and the partial sums are added in group-chunk order; used for the
    multi-core CPU baseline."""
    J = len(terms.x)

    def part(js):
        acc = np.zeros_like(vec)
        for j in js:
            src = xsource_sortmerge(states, terms.x[j])
            acc = acc + gather_fill(vec, src) * diagonal(states, terms.z[j], terms.c[j])
        return acc

    if threads <= 1:
        return part(range(J))
    chunks = [range(a, min(J, a + (J + threads - 1) // threads))
              for a in range(0, J, (J + threads - 1) // threads)]
    with ThreadPoolExecutor(max_workers=threads) as pool:
        parts = list(pool.map(part, chunks))
    out = np.zeros_like(vec)
    for p in parts:
        out = out + p
    return out


def initial_vector(terms: OracleTerms, states):
    """run_sqd's vinit, sqd.py:373-398: one-hot at the first minimum of the x=0 group's diagonal
    when group 0 is diagonal, else one-hot at index 0; dtype of the phased coefficients."""
    D = len(states)
    v = np.zeros(D, dtype=terms.c.dtype)
    if terms.x[0] == 0:
        d0 = np.real(diagonal(states, terms.z[0], terms.c[0]))
        v[int(np.argmin(d0))] = 1
    else:
        v[0] = 1
    return v


def prepare(hamiltonian, states):
    """Front half of sqd(), sqd.py:222-237 + 316: terms (force_real=True) and the sorted unique
    subspace.  ``states`` is either (D_in, n) 0/1 rows (duplicates allowed) or 1-d uint64."""
    if isinstance(hamiltonian, OracleTerms):
        terms = hamiltonian
    else:
        terms = from_paulisum(hamiltonian, force_real=True)
    states = np.asarray(states)
    if states.ndim == 2:
        S = uniquify(pack_states(states))
    else:
        S = uniquify(states.astype(np.uint64))
    return terms, S


def sqd(hamiltonian, states, states_size=None, return_eigvec=True, maxiter=1000, tol=None):
    """sqd(), sqd.py:181-248, default cache_level=(1, 0).

    ``states_size`` (sqd.py:222-225) pads the reference's vectors with inert fill rows; its only
    observable effect is the vector length in the convergence test (ground_locg.py:330), which is
    reproduced through ``tol_dim``.  Returns (eigval, eigvec, basis_states[, niter])."""
    n_in = np.asarray(states).shape[0]
    if states_size is None:
        states_size = n_in
    if states_size < n_in:
        raise ValueError('states_size smaller than the states array length')
    terms, S = prepare(hamiltonian, states)
    xs = xsources_all(S, terms)
    vinit = initial_vector(terms, S)
    eigval, eigvec, niter = ground_locg(lambda v: matvec_xcached(v, xs, terms, S), vinit,
                                        maxiter=maxiter, tol=tol, tol_dim=states_size)
    if not return_eigvec:
        return float(eigval)
    return float(eigval), eigvec, unpack_states(S, terms.num_qubits), niter


def hproj_dense(terms: OracleTerms, states):
    """Dense projected matrix from the grouped form: H[i, xsource_j[i]] += diag_j[i].  (The
    reference's ``hproj``, sqd.py:251-296, packs the states without the padding bit its padded
    Hamiltonian expects; this builds the matrix the SQD matvec applies.)"""
    D = len(states)
    H = np.zeros((D, D), dtype=np.complex128)
    for j in range(len(terms.x)):
        src = xsource_search(states, terms.x[j])
        d = diagonal(states, terms.z[j], terms.c[j])
        rows = np.nonzero(src >= 0)[0]
        H[rows, src[rows]] += d[rows]
    return H
