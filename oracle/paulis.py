"""Oracle restatement of ``PauliSumXZ.from_paulisum`` (``rqutils/paulis/symplectic.py:51-125``).

Written with plain Python containers on purpose (it is a checker, independent of the vectorised
host code in ``rqutils_gb300.paulis``).  Test infrastructure only.
"""
from dataclasses import dataclass
import warnings

import numpy as np

# (-i)^k for k = popcount(x & z) mod 4 -- symplectic.py:109-111
_PHASES = (1.0 + 0.0j, -1.0j, -1.0 + 0.0j, 1.0j)


@dataclass
class OracleTerms:
    """Pauli sum grouped by X signature.

    ``x[j]`` is the X mask of group ``j`` (groups in ascending order of the mask, which is the order
    ``np.unique`` gives the reference's bool rows, symplectic.py:99); ``z[j, k]`` / ``c[j, k]`` are the
    Z masks and phased coefficients of its terms in the order of the consolidated string list, padded
    with ``z = 0, c = 0`` up to the largest group (symplectic.py:102-112).
    """
    x: np.ndarray        # (J,) uint64
    z: np.ndarray        # (J, Kmax) uint64
    c: np.ndarray        # (J, Kmax) float64 or complex128
    counts: np.ndarray   # (J,) int -- number of real (unpadded) terms per group
    num_qubits: int

    def to_reference_packed(self, add_padding=False):
        """The reference's packed uint8 arrays ``(x (J,B), z (J,Kmax,B))`` -- symplectic.py:117-124."""
        n = self.num_qubits
        ncol = n + (1 if add_padding else 0)

        def bits(masks):
            masks = np.asarray(masks, dtype=np.uint64)
            cols = np.zeros(masks.shape + (ncol,), dtype=np.uint8)
            for q in range(n):
                col = ncol - 1 - q
                cols[..., col] = ((masks >> np.uint64(q)) & np.uint64(1)).astype(np.uint8)
            return np.packbits(cols, axis=-1)

        return bits(self.x), bits(self.z)


def _mask_from_string(s, letters):
    n = len(s)
    m = 0
    for col, ch in enumerate(s):
        if ch in letters:
            m |= 1 << (n - 1 - col)
    return m


def from_paulisum(paulisum, force_real=False):
    """Restates symplectic.py:58-115 for the ``([strings], [coeffs])`` input form.

    Steps: length checks (60-63); drop exactly-zero coefficients (68-70); merge duplicate strings,
    summing their coefficients, in lexicographic string order (71-73); X bits = X|Y, Z bits = Y|Z
    (74-75); optional real cast with a warning (93-96); group by X mask in ascending order (99);
    phase each coefficient by (-i)^{popcount(x&z) mod 4} (109-112); real dtype if every phased
    coefficient is real (114-115).
    """
    if not isinstance(paulisum, tuple):
        raise ValueError('Unsupported input type')
    paulis, coeffs = paulisum
    if len(paulis) != len(coeffs):
        raise ValueError('Lengths of Pauli and coeff lists do not match')
    if len(set(len(p) for p in paulis)) != 1:
        raise ValueError('Pauli strings have non-uniform lengths')
    coeffs = np.array(coeffs)
    n = len(paulis[0])

    merged = {}
    for p, cf in zip(paulis, coeffs):
        if cf == 0:
            continue
        key = p.upper()
        merged[key] = merged.get(key, 0) + cf
    strings = sorted(merged)
    vals = np.array([merged[s] for s in strings], dtype=coeffs.dtype)

    if force_real:
        if np.any(np.imag(vals) != 0.):
            warnings.warn('Found nonzero imaginary part when force_real=True')
        vals = np.real(vals).copy()

    xm = [_mask_from_string(s, 'XY') for s in strings]
    zm = [_mask_from_string(s, 'YZ') for s in strings]
    groups = {}
    for s_idx, xv in enumerate(xm):
        groups.setdefault(xv, []).append(s_idx)
    xkeys = sorted(groups)
    kmax = max(len(v) for v in groups.values())
    J = len(xkeys)
    x = np.array(xkeys, dtype=np.uint64)
    z = np.zeros((J, kmax), dtype=np.uint64)
    c = np.zeros((J, kmax), dtype=np.complex128)
    counts = np.zeros(J, dtype=np.int64)
    for j, xv in enumerate(xkeys):
        members = groups[xv]
        counts[j] = len(members)
        for k, s_idx in enumerate(members):
            z[j, k] = zm[s_idx]
            c[j, k] = vals[s_idx] * _PHASES[bin(xv & zm[s_idx]).count('1') & 3]
    if np.all(c.imag == 0.):
        c = c.real.copy()
    return OracleTerms(x=x, z=z, c=c, counts=counts, num_qubits=n)


def from_reference_arrays(x_packed, z_packed, c, num_qubits, padded):
    """Build OracleTerms from the reference's packed arrays (PauliSumXZ.x / .z / .c)."""
    n = num_qubits
    ncol = n + (1 if padded else 0)

    def masks(packed):
        bits = np.unpackbits(np.asarray(packed, dtype=np.uint8), axis=-1)[..., :ncol]
        out = np.zeros(bits.shape[:-1], dtype=np.uint64)
        for q in range(n):
            out |= bits[..., ncol - 1 - q].astype(np.uint64) << np.uint64(q)
        return out

    x = masks(x_packed)
    z = masks(z_packed)
    c = np.asarray(c)
    counts = np.array([int(np.count_nonzero(row)) for row in c])
    return OracleTerms(x=x, z=z, c=c.copy(), counts=counts, num_qubits=n)
