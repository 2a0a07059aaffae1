"""Seeded synthetic workloads for the SQD path: Pauli sums and sampled bitstring subspaces.

The reference publishes no dataset or benchmark inputs; these generators produce inputs with the
shapes and value distributions of the benchmark configurations:

* ``random_pauli_sum``  -- K terms, locality uniform in [lo, hi], support qubits uniform without
  replacement, each support Pauli uniform in {X, Y, Z}, coefficients N(0, 1);
* ``hubbard_jw``        -- Fermi-Hubbard model on an Lx x Ly lattice, Jordan-Wigner mapped;
* ``chemistry_jw``      -- random two-body "chemistry-shaped" Hamiltonian, Jordan-Wigner mapped;
* ``sample_sector``     -- D distinct bitstrings drawn uniformly from a fixed-Hamming-weight sector
  (optionally a product of sectors, e.g. N_up electrons in the up-spin orbitals and N_down in the
  down-spin orbitals), returned sorted as uint64 (bit q = qubit q).

String convention (shared with rqutils): character 0 of a Pauli string acts on qubit n-1.
"""
import numpy as np


# ----------------------------------------------------------------------------------------------
# Pauli sums
# ----------------------------------------------------------------------------------------------

def random_pauli_sum(rng, n, K, locality=(1, 4)):
    """Random real Pauli sum: returns ([str] * K, float64 (K,))."""
    lo, hi = locality
    chars = np.array(list('XYZ'))
    paulis = []
    for _ in range(K):
        w = int(rng.integers(lo, hi + 1))
        support = rng.choice(n, size=w, replace=False)
        row = np.full(n, 'I')
        row[n - 1 - support] = chars[rng.integers(0, 3, size=w)]
        paulis.append(''.join(row))
    coeffs = rng.normal(0., 1., size=K)
    return paulis, coeffs


def _string(n, ops):
    """Pauli string of length n from {qubit: 'X'|'Y'|'Z'}."""
    row = ['I'] * n
    for q, p in ops.items():
        row[n - 1 - q] = p
    return ''.join(row)


def hubbard_sites(Lx, Ly, periodic=True):
    """Nearest-neighbour bonds (i, j), i < j, of an Lx x Ly lattice; site = x + Lx * y."""
    bonds = set()
    for y in range(Ly):
        for x in range(Lx):
            i = x + Lx * y
            for dx, dy in ((1, 0), (0, 1)):
                xx, yy = x + dx, y + dy
                if periodic:
                    xx %= Lx
                    yy %= Ly
                elif xx >= Lx or yy >= Ly:
                    continue
                j = xx + Lx * yy
                if i != j:
                    bonds.add((min(i, j), max(i, j)))
    return sorted(bonds)


def hubbard_jw(Lx=4, Ly=4, t=1.0, U=4.0, periodic=True):
    """Jordan-Wigner mapped Fermi-Hubbard Hamiltonian.

    H = -t sum_{<ij>, s} (a+_{is} a_{js} + h.c.) + U sum_i n_{i,up} n_{i,down}.
    Spin-orbital ordering: qubit i is (site i, up), qubit Ns + i is (site i, down), Ns = Lx * Ly.
    Hopping p < q maps to -t/2 (X_p Z..Z X_q + Y_p Z..Z Y_q) with Z on every qubit strictly
    between p and q; n_p n_q maps to (I - Z_p - Z_q + Z_p Z_q) / 4.  Returns ([str], float64).
    """
    Ns = Lx * Ly
    n = 2 * Ns
    terms = {}

    def add(label, c):
        terms[label] = terms.get(label, 0.) + c

    for (i, j) in hubbard_sites(Lx, Ly, periodic):
        for off in (0, Ns):
            p, q = i + off, j + off
            chain = {k: 'Z' for k in range(p + 1, q)}
            add(_string(n, {**chain, p: 'X', q: 'X'}), -0.5 * t)
            add(_string(n, {**chain, p: 'Y', q: 'Y'}), -0.5 * t)
    for i in range(Ns):
        up, dn = i, Ns + i
        add(_string(n, {}), U / 4.)
        add(_string(n, {up: 'Z'}), -U / 4.)
        add(_string(n, {dn: 'Z'}), -U / 4.)
        add(_string(n, {up: 'Z', dn: 'Z'}), U / 4.)
    labels = sorted(terms)
    return labels, np.array([terms[k] for k in labels])


# ----------------------------------------------------------------------------------------------
# Symplectic products, for the Jordan-Wigner mapping of ladder-operator products
# ----------------------------------------------------------------------------------------------

def _ladder(p, dagger):
    """JW ladder operator on qubit p as two (x, z, coeff) Pauli terms:
    a_p = Z_0..Z_{p-1} (X_p + i Y_p) / 2,  a+_p = Z_0..Z_{p-1} (X_p - i Y_p) / 2,
    with Y = i X Z in the symplectic form P(x, z) = i^{x.z} X^x Z^z (Hermitian convention)."""
    chain = (1 << p) - 1
    xb = 1 << p
    sgn = -1.0 if dagger else 1.0
    # X_p: x = xb, z = chain ; i*Y_p: x = xb, z = chain | xb, coefficient i * sgn
    return [(xb, chain, 0.5 + 0j), (xb, chain | xb, 0.5j * sgn)]


def _popcount(a):
    return bin(a).count('1')


def _mul(t1, t2):
    """Product of Hermitian-convention Pauli terms P(x1,z1) P(x2,z2), both with phase i^{x.z}."""
    x1, z1, c1 = t1
    x2, z2, c2 = t2
    # P(x,z) = i^{|x&z|} X^x Z^z ; X^x1 Z^z1 X^x2 Z^z2 = (-1)^{|z1&x2|} X^{x1^x2} Z^{z1^z2}
    x, z = x1 ^ x2, z1 ^ z2
    k = _popcount(x1 & z1) + _popcount(x2 & z2) + 2 * _popcount(z1 & x2) - _popcount(x & z)
    return (x, z, c1 * c2 * (1j ** (k % 4)))


def _label(n, x, z):
    row = []
    for col in range(n):
        q = n - 1 - col
        xb, zb = (x >> q) & 1, (z >> q) & 1
        row.append('IXZY'[xb | (zb << 1)] if not (xb and zb) else 'Y')
    return ''.join(row)


def chemistry_jw(n_spatial, rng, keep=None, h_scale=None, g_scale=0.1):
    """Random "chemistry-shaped" Hamiltonian, Jordan-Wigner mapped.

    One-body h_pq ~ N(0, 1/n_spatial) symmetric; two-body (pq|rs) ~ N(0, g_scale^2) with 8-fold
    symmetry; H = sum_{pq,s} h_pq a+_{ps} a_{qs} + 1/2 sum_{pqrs,s,t} (pq|rs) a+_{ps} a+_{rt} a_{st} a_{qs}.
    Spin-orbital ordering: qubit p is (p, alpha), qubit n_spatial + p is (p, beta).  The qubit
    Hamiltonian keeps its ``keep`` largest-|c| Pauli terms (all if None).  Returns ([str], float64).
    The mapping runs in pure Python over the ladder-operator expansions, so it is meant for small
    n_spatial in tests; ``chemistry_terms_fast`` handles the benchmark size.
    """
    ns = n_spatial
    n = 2 * ns
    if h_scale is None:
        h_scale = 1.0 / np.sqrt(ns)
    h = rng.normal(0., h_scale, size=(ns, ns))
    h = 0.5 * (h + h.T)
    g = _random_eri(rng, ns, g_scale)
    acc = {}

    def add_product(ops, coeff):
        terms = [(0, 0, complex(coeff))]
        for (p, dag) in ops:
            terms = [_mul(a, b) for a in terms for b in _ladder(p, dag)]
        for (x, z, c) in terms:
            acc[(x, z)] = acc.get((x, z), 0) + c

    for s in (0, ns):
        for p in range(ns):
            for q in range(ns):
                if h[p, q] != 0:
                    add_product([(p + s, True), (q + s, False)], h[p, q])
    for s in (0, ns):
        for t in (0, ns):
            for p in range(ns):
                for q in range(ns):
                    for r in range(ns):
                        for u in range(ns):
                            if p + s == r + t or q + s == u + t:
                                continue
                            add_product([(p + s, True), (r + t, True), (u + t, False),
                                         (q + s, False)], 0.5 * g[p, q, r, u])
    items = [(k, v) for k, v in acc.items() if abs(v) > 1e-14]
    # Hermitian-convention coefficients of a Hermitian operator are real
    labels = [_label(n, x, z) for (x, z), _ in items]
    coeffs = np.array([v.real for _, v in items])
    order = np.argsort(-np.abs(coeffs), kind='stable')
    if keep is not None:
        order = order[:keep]
    return [labels[i] for i in order], coeffs[order]


def _random_eri(rng, ns, scale):
    """(pq|rs) ~ N(0, scale^2) with the 8-fold permutational symmetry of real orbitals."""
    g = rng.normal(0., scale, size=(ns, ns, ns, ns))
    g = g + g.transpose(1, 0, 2, 3)
    g = g + g.transpose(0, 1, 3, 2)
    g = g + g.transpose(2, 3, 0, 1)
    return g / 8.0


# ----------------------------------------------------------------------------------------------
# Subspace sampling
# ----------------------------------------------------------------------------------------------

def _fixed_weight_words(rng, nbits, weight, count):
    """``count`` uniform random nbits-bit words (nbits <= 32) with popcount == weight."""
    out = []
    have = 0
    while have < count:
        need = count - have
        batch = max(1024, int(need * 1.2 * (2 ** nbits) / max(1, _comb(nbits, weight))))
        batch = min(batch, 1 << 24)
        w = rng.integers(0, 1 << nbits, size=batch, dtype=np.uint64)
        w = w[np.bitwise_count(w) == weight]
        out.append(w[:need])
        have += len(out[-1])
    return np.concatenate(out)


def _comb(n, k):
    from math import comb
    return comb(n, k)


def sample_sector(rng, D, blocks):
    """D distinct states drawn uniformly without replacement from a product of fixed-weight blocks.

    ``blocks`` is a list of (nbits, weight), least significant block first; e.g. the 8-up/8-down
    sector of 32 spin-orbitals is ``[(16, 8), (16, 8)]`` and 10 of 20 qubits is ``[(20, 10)]``.
    Blocks wider than 32 bits are split into two halves of the word, which is only uniform when the
    caller asks for a product sector, so widths above 32 are rejected.  Returns sorted uint64 (D,).
    """
    total = 1
    for nb, w in blocks:
        if nb > 32:
            raise ValueError('sector blocks are limited to 32 bits; split wider ones')
        total *= _comb(nb, w)
    if D > total:
        raise ValueError(f'D={D} exceeds the sector size {total}')
    if D > total // 2:
        # dense: enumerate the sector and choose without replacement
        allst = _enumerate_sector(blocks)
        return np.sort(rng.choice(allst, size=D, replace=False))
    have = np.zeros(0, dtype=np.uint64)
    while len(have) < D:
        need = int((D - len(have)) * 1.05) + 16
        words = np.zeros(need, dtype=np.uint64)
        shift = 0
        for nb, w in blocks:
            words |= _fixed_weight_words(rng, nb, w, need) << np.uint64(shift)
            shift += nb
        have = np.unique(np.concatenate([have, words]))
    # drop a uniformly chosen surplus
    if len(have) > D:
        have = np.sort(rng.choice(have, size=D, replace=False))
    return have


def _enumerate_sector(blocks):
    parts = []
    for nb, w in blocks:
        allw = np.arange(1 << nb, dtype=np.uint64)
        parts.append(allw[np.bitwise_count(allw) == w])
    out = parts[0]
    shift = blocks[0][0]
    for (nb, _), part in zip(blocks[1:], parts[1:]):
        out = (out[:, None] | (part[None, :] << np.uint64(shift))).ravel()
        shift += nb
    return np.sort(out)


def random_vector(rng, D, complex_=True, dtype=np.complex128):
    """Normalised complex-normal (or real normal) vector."""
    if complex_:
        v = rng.normal(size=D) + 1j * rng.normal(size=D)
    else:
        v = rng.normal(size=D)
    v = v / np.linalg.norm(v)
    return v.astype(dtype)
