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


def random_pauli_masks(rng, n, K, locality=(1, 4)):
    """Vectorised random real Pauli sum: K terms of weight uniform in ``locality`` on distinct
    random qubits, letters uniform in X/Y/Z, coefficients N(0, 1).  Returns ([str] * K, (K,))."""
    lo, hi = locality
    w = rng.integers(lo, hi + 1, size=K)
    order = np.argsort(rng.random((K, n)), axis=1)          # a random permutation per term
    pick = np.arange(n)[None, :] < w[:, None]                  # its first w qubits
    letter = rng.integers(1, 4, size=(K, n))                  # 1 = X, 2 = Z, 3 = Y
    bit = np.left_shift(np.uint64(1), order.astype(np.uint64))
    xb = np.where(pick & (letter != 2), bit, np.uint64(0))
    zb = np.where(pick & (letter != 1), bit, np.uint64(0))
    x = np.bitwise_or.reduce(xb, axis=1)
    z = np.bitwise_or.reduce(zb, axis=1)
    return xz_labels(x, z, n), rng.normal(0., 1., size=K)


def batched_random_problems(seed, P=256, n_range=(16, 40), k_range=(100, 2000),
                            d_range=(2 ** 10, 2 ** 18)):
    """P independent random Pauli-sum SQD problems: N uniform in ``n_range``, K log-uniform in
    ``k_range``, D log-uniform in ``d_range`` (capped at half the sector), states of Hamming
    weight N // 2 (one block for N <= 32; above, a product of two half-width blocks).  Returns
    (paulisums [(labels, coeffs)], states [sorted uint64], nqubits)."""
    rng = np.random.default_rng(seed)
    hams, states, ns = [], [], []
    for _ in range(P):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        K = int(np.exp(rng.uniform(np.log(k_range[0]), np.log(k_range[1]))))
        D = int(np.exp(rng.uniform(np.log(d_range[0]), np.log(d_range[1]))))
        w = n // 2
        if n <= 32:
            blocks = [(n, w)]
        else:
            blocks = [(n // 2, w // 2), (n - n // 2, w - w // 2)]
        total = 1
        for nb, ww in blocks:
            total *= _comb(nb, ww)
        D = max(1, min(D, total // 2))
        hams.append(random_pauli_masks(rng, n, K))
        states.append(sample_sector(rng, D, blocks))
        ns.append(n)
    return hams, states, ns


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
# Jordan-Wigner mapping of ladder-operator products (symplectic form)
# ----------------------------------------------------------------------------------------------

def chemistry_jw(n_spatial, rng, keep=None, h_scale=None, g_scale=0.1, chunk=1 << 18):
    """Random "chemistry-shaped" Hamiltonian, Jordan-Wigner mapped.

    One-body h_pq ~ N(0, h_scale^2) symmetric (default h_scale^2 = 1 / n_spatial); two-body
    (pq|rs) ~ N(0, g_scale^2) with the 8-fold symmetry of real orbitals;
    H = sum_{pq,s} h_pq a+_{ps} a_{qs} + 1/2 sum_{pqrs,s,t} (pq|rs) a+_{ps} a+_{rt} a_{st} a_{qs}.
    Spin-orbital ordering: qubit p is (p, alpha), qubit n_spatial + p is (p, beta).  The
    ladder-operator products are expanded in the symplectic form, vectorised over index tuples
    and aggregated by sorting; the ``keep`` largest-|c| Pauli terms are returned (all if None).
    Returns ([str], float64).
    """
    ns = n_spatial
    n = 2 * ns
    if n > 64:
        raise ValueError('at most 32 spatial orbitals (64 qubits)')
    if h_scale is None:
        h_scale = 1.0 / np.sqrt(ns)
    h = rng.normal(0., h_scale, size=(ns, ns))
    h = 0.5 * (h + h.T)
    g = _random_eri(rng, ns, g_scale)
    acc_x, acc_z, acc_c = [], [], []

    def flush(xs, zs, cs):
        x, z, c = _aggregate(np.concatenate(xs), np.concatenate(zs), np.concatenate(cs))
        acc_x.append(x)
        acc_z.append(z)
        acc_c.append(c)

    # one-body: a+_p a_q within a spin block
    pp, qq = np.meshgrid(np.arange(ns), np.arange(ns), indexing='ij')
    pp, qq = pp.ravel(), qq.ravel()
    cf = h[pp, qq]
    xs, zs, cs = [], [], []
    for off in (0, ns):
        x, z, c = _ladder_product([(pp + off, True), (qq + off, False)], cf)
        xs.append(x), zs.append(z), cs.append(c)
    flush(xs, zs, cs)
    # two-body: 1/2 (pq|rs) a+_{p s} a+_{r t} a_{s t} a_{q s}
    idx = np.arange(ns ** 4)
    P, Q, Rr, Ss = np.unravel_index(idx, (ns, ns, ns, ns))
    G = 0.5 * g[P, Q, Rr, Ss]
    for so in (0, ns):
        for to in (0, ns):
            a, b, cc, d = P + so, Rr + to, Ss + to, Q + so
            ok = (a != b) & (cc != d)
            a, b, cc, d, Gk = a[ok], b[ok], cc[ok], d[ok], G[ok]
            for lo in range(0, len(a), chunk):
                sl = slice(lo, lo + chunk)
                x, z, c = _ladder_product([(a[sl], True), (b[sl], True), (cc[sl], False),
                                           (d[sl], False)], Gk[sl])
                flush([x], [z], [c])
    x, z, c = _aggregate(np.concatenate(acc_x), np.concatenate(acc_z), np.concatenate(acc_c))
    # Hermitian operator: the Pauli coefficients are real up to round-off
    c = c.real
    nz = np.abs(c) > 1e-13
    x, z, c = x[nz], z[nz], c[nz]
    order = np.argsort(-np.abs(c), kind='stable')
    if keep is not None:
        order = order[:keep]
    return xz_labels(x[order], z[order], n), c[order]


def _popcount64(a):
    return np.bitwise_count(a).astype(np.int64)


def _ladder_product(ops, coeff):
    """Expand prod_k (ladder op k) * coeff for arrays of tuples.  Ladder operators on qubit p:
    a_p = Z_0..Z_{p-1} (X_p + i Y_p) / 2, a+_p = Z_0..Z_{p-1} (X_p - i Y_p) / 2, written with
    Hermitian Pauli strings P(x, z) = i^{|x & z|} X^x Z^z.  Returns flat (x, z, c) arrays."""
    one = np.uint64(1)
    x = np.zeros((len(coeff), 1), dtype=np.uint64)
    z = np.zeros((len(coeff), 1), dtype=np.uint64)
    c = np.asarray(coeff, dtype=np.complex128)[:, None]
    for p, dagger in ops:
        p = np.asarray(p, dtype=np.uint64)
        xb = one << p
        chain = xb - one
        # the two terms of the ladder operator: (xb, chain, 1/2) and (xb, chain|xb, +-i/2)
        tx = np.stack([xb, xb], axis=1)
        tz = np.stack([chain, chain | xb], axis=1)
        tc = np.array([0.5, (-0.5j if dagger else 0.5j)])
        X1, Z1 = x[:, :, None], z[:, :, None]
        X2, Z2 = tx[:, None, :], tz[:, None, :]
        Xn, Zn = X1 ^ X2, Z1 ^ Z2
        k = (_popcount64(X1 & Z1) + _popcount64(X2 & Z2) + 2 * _popcount64(Z1 & X2)
             - _popcount64(Xn & Zn)) & 3
        ph = np.array([1, 1j, -1, -1j])[k]
        c = (c[:, :, None] * tc[None, None, :] * ph).reshape(len(c), -1)
        x = Xn.reshape(len(c), -1)
        z = Zn.reshape(len(c), -1)
    return x.ravel(), z.ravel(), c.ravel()


def _aggregate(x, z, c):
    """Sum coefficients of equal (x, z) strings (sorted by (x, z))."""
    if len(x) == 0:
        return x, z, c
    order = np.lexsort((z, x))
    x, z, c = x[order], z[order], c[order]
    start = np.concatenate([[True], (x[1:] != x[:-1]) | (z[1:] != z[:-1])])
    idx = np.nonzero(start)[0]
    return x[idx], z[idx], np.add.reduceat(c, idx)


def xz_labels(x, z, n):
    """Pauli labels of (x, z) masks; character 0 is qubit n-1."""
    x = np.asarray(x, dtype=np.uint64)
    z = np.asarray(z, dtype=np.uint64)
    shifts = np.arange(n - 1, -1, -1, dtype=np.uint64)
    xb = ((x[:, None] >> shifts) & np.uint64(1)).astype(np.uint8)
    zb = ((z[:, None] >> shifts) & np.uint64(1)).astype(np.uint8)
    code = xb + 2 * zb  # I=0, X=1, Z=2, Y=3
    chars = np.array([ord('I'), ord('X'), ord('Z'), ord('Y')], dtype=np.uint32)[code]
    return [s for s in np.ascontiguousarray(chars).view(f'<U{n}').ravel()]


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
        have = sorted_unique(np.concatenate([have, words]))
    # drop a uniformly chosen surplus (keeps the array sorted)
    if len(have) > D:
        have = np.delete(have, rng.choice(len(have), size=len(have) - D, replace=False))
    return have


def low_double_occupancy_states(rng, D, Ns=16, n_up=None, n_dn=None):
    """D distinct half-filled Hubbard configurations with at most one doubly occupied site, drawn
    uniformly without replacement and sorted (bit i = site i up, bit Ns + i = site i down).  With
    n_up = n_dn = Ns / 2 the pool is C(Ns, Ns/2) (1 + (Ns/2)^2) states (836,550 for 4x4); the
    hopping terms connect a large part of it, unlike a uniform sample of the whole sector."""
    n_up = Ns // 2 if n_up is None else n_up
    n_dn = Ns - n_up if n_dn is None else n_dn
    if n_up + n_dn != Ns:
        raise ValueError('half filling: n_up + n_dn must equal the number of sites')
    full = (1 << Ns) - 1
    ups = _enumerate_sector([(Ns, n_up)])
    comp = (~ups) & np.uint64(full)                 # down = complement: no double occupancy
    pools = [ups | (comp << np.uint64(Ns))]
    # one double: move one down electron from a hole of the up pattern onto an up site
    bits = np.arange(Ns, dtype=np.uint64)
    for a in range(Ns):
        for b in range(Ns):
            sel = ((ups >> bits[a]) & np.uint64(1)).astype(bool) & \
                  ((comp >> bits[b]) & np.uint64(1)).astype(bool)
            dn = (comp[sel] | (np.uint64(1) << bits[a])) & ~(np.uint64(1) << bits[b])
            pools.append(ups[sel] | (dn << np.uint64(Ns)))
    pool = np.concatenate(pools)
    if D > len(pool):
        raise ValueError(f'D={D} exceeds the pool of {len(pool)} configurations')
    return np.sort(rng.choice(pool, size=D, replace=False))


def sorted_unique(a):
    """Sorted distinct values of a 1-d array (sort + adjacent difference)."""
    a = np.sort(np.asarray(a))
    if len(a) == 0:
        return a
    keep = np.empty(len(a), dtype=bool)
    keep[0] = True
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


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


class BenchmarkProblem:
    """One benchmark configuration: the Pauli sum, the sorted subspace and the seeded input vector.

    ``name``: ``hubbard`` (Fermi-Hubbard 4x4 periodic, t = 1, U = 4, 32 spin-orbitals; D = 2^20
    drawn from the 8-up / 8-down sector, seed 1; complex64), ``chemistry`` (32 spatial orbitals ->
    64 spin-orbitals, the 50,000 largest |c|; D = 2^26 at 16 alpha + 16 beta, seed 5; complex64) or
    ``random20`` (20 qubits, K = 200 terms of locality 1..4, N(0, 1) coefficients; D = 16384 at
    Hamming weight 10, seed 20; complex128).  ``rows`` overrides D (smaller profiling cases)."""

    def __init__(self, name, rows=None):
        self.name = name
        if name == 'hubbard':
            self.paulis, self.coeffs = hubbard_jw(4, 4, 1.0, 4.0, periodic=True)
            self.D, self.seed = 1 << 20, 1
            self.blocks = [(16, 8), (16, 8)]
            self.vtype = 'c64'
            self.label = 'hubbard4x4_periodic_t1_U4_jw32_D1048576_sector8u8d'
            self.lobpcg = True
        elif name == 'chemistry':
            self.paulis, self.coeffs = chemistry_jw(32, np.random.default_rng(4), keep=50000)
            self.D, self.seed = 1 << 26, 5
            self.blocks = [(32, 16), (32, 16)]
            self.vtype = 'c64'
            self.label = 'chemistry32orb_jw64_K50000_D67108864_sector16a16b'
            self.lobpcg = False
        elif name == 'random20':
            self.paulis, self.coeffs = random_pauli_sum(np.random.default_rng(20), 20, 200)
            self.D, self.seed = 16384, 20
            self.blocks = [(20, 10)]
            self.vtype = 'c128'
            self.label = 'random20_K200_loc1to4_D16384_weight10'
            self.lobpcg = True
        else:
            raise ValueError(f'unknown workload {name}')
        if rows:
            self.D = int(rows)
            self.label += f'_rows{self.D}'
        self.num_qubits = sum(nb for nb, _ in self.blocks)
        self.S = sample_sector(np.random.default_rng(self.seed), self.D, self.blocks)
        self.x = random_vector(np.random.default_rng(self.seed + 1), self.D, complex_=True)


def random_vector(rng, D, complex_=True, dtype=np.complex128):
    """Normalised complex-normal (or real normal) vector."""
    if complex_:
        v = rng.normal(size=D) + 1j * rng.normal(size=D)
    else:
        v = rng.normal(size=D)
    v = v / np.linalg.norm(v)
    return v.astype(dtype)
