r"""Symplectic (XZ) representation of Pauli sums -- mirror of ``rqutils.paulis.symplectic``.

A Pauli string Q over n qubits is :math:`Q = (-i)^{x \cdot z} Z^{z} X^{x}` with X signature x and Z
signature z (``rqutils/paulis/symplectic.py:11-19``).  ``PauliSumXZ`` groups the terms of a sum by
X signature, with each coefficient multiplied by :math:`(-i)^{x \cdot z \bmod 4}`.

Compared with the reference, the arrays are held in a compact grouped form (one uint64 mask per
signature, bit q = qubit q, n <= 64): ``xmask (J,)``, ``toff (J+1,)``, ``zmask (K,)``,
``coef (K,)``.  The reference's padded packed arrays ``x (J, B)``, ``z (J, Kmax, B)``,
``c (J, Kmax)`` are produced on demand (properties ``x``, ``z``, ``c``, ``arrays``), so a
Hamiltonian with a few large groups does not pay ``J * Kmax`` memory.  ``matmul`` runs on the GPU.
"""
import warnings

import numpy as np

_PHASES = np.array([1., -1.j, -1., 1.j])


def _is_sparse_pauli_op(obj):
    try:
        from qiskit.quantum_info import SparsePauliOp
    except ImportError:
        return False
    return isinstance(obj, SparsePauliOp)


def bits_to_masks(bits):
    """(..., n) bool, column 0 = qubit n-1  ->  (...,) uint64 with bit q = qubit q."""
    bits = np.asarray(bits, dtype=bool)
    n = bits.shape[-1]
    if n > 64:
        raise ValueError('at most 64 qubits are supported')
    w = np.left_shift(np.uint64(1), np.arange(n - 1, -1, -1, dtype=np.uint64))
    return np.bitwise_or.reduce(np.where(bits, w, np.uint64(0)), axis=-1).astype(np.uint64) \
        if n else np.zeros(bits.shape[:-1], dtype=np.uint64)


def masks_to_packed(masks, n, padded):
    """uint64 masks -> the reference's packed big-endian bytes, with the optional leading zero
    padding bit (symplectic.py:117-124)."""
    masks = np.asarray(masks, dtype=np.uint64)
    ncol = n + (1 if padded else 0)
    shifts = np.arange(ncol - 1, -1, -1, dtype=np.uint64)
    cols = ((masks[..., None] >> shifts) & np.uint64(1)).astype(np.uint8)
    if padded:
        cols[..., 0] = 0
    return np.packbits(cols, axis=-1)


def packed_to_masks(packed, n, padded):
    """Inverse of masks_to_packed (the padding bit, if any, is dropped)."""
    ncol = n + (1 if padded else 0)
    bits = np.unpackbits(np.asarray(packed, dtype=np.uint8), axis=-1)[..., :ncol]
    if padded:
        bits = bits[..., 1:]
    return bits_to_masks(bits.astype(bool))


class PauliSumXZ:
    """Symplectic (XZ) representation of a sum of Pauli strings (symplectic.py:42-49).

    ``PauliSumXZ(x, z, c, num_qubits)`` accepts the reference's packed arrays; the padding bit is
    detected from the byte count when unambiguous and otherwise assumed present when
    ``padded=None`` (``sqd`` requires the padded form, as in the reference).
    """

    def __init__(self, x, z, c, num_qubits, padded=None):
        x = np.asarray(x, dtype=np.uint8)
        z = np.asarray(z, dtype=np.uint8)
        c = np.asarray(c)
        n = int(num_qubits)
        if padded is None:
            # the byte count decides when n % 8 == 0; otherwise both forms have the same size and
            # the padded form (the one sqd() requires) is assumed
            bu, bp = (n + 7) // 8, (n + 8) // 8
            padded = True if bu == bp else (x.shape[-1] == bp)
        self.num_qubits = n
        self.padded = bool(padded)
        self._packed = (x, z, c)
        xm = packed_to_masks(x, n, self.padded)
        zm = packed_to_masks(z, n, self.padded)
        counts = np.array([_trimmed_len(row) for row in c], dtype=np.int64)
        toff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.xmask = xm
        self.toff = toff
        self.zmask = np.concatenate([zm[j, :counts[j]] for j in range(len(counts))]) \
            if len(counts) else np.zeros(0, np.uint64)
        self.coef = np.concatenate([c[j, :counts[j]] for j in range(len(counts))]) \
            if len(counts) else np.zeros(0, c.dtype)

    @classmethod
    def _from_compact(cls, xmask, toff, zmask, coef, num_qubits, padded):
        obj = cls.__new__(cls)
        obj.num_qubits = int(num_qubits)
        obj.padded = bool(padded)
        obj.xmask = np.asarray(xmask, dtype=np.uint64)
        obj.toff = np.asarray(toff, dtype=np.int64)
        obj.zmask = np.asarray(zmask, dtype=np.uint64)
        obj.coef = np.asarray(coef)
        obj._packed = None
        return obj

    # ------------------------------------------------------------------------------------------
    @classmethod
    def from_paulisum(cls, paulisum, force_real=False, add_padding=False, device=None):
        """symplectic.py:51-125: parse ``([str], [coeff])`` or a qiskit ``SparsePauliOp``;
        consolidate (drop exact zeros, merge duplicate strings in lexicographic order); group by X
        signature in ascending order; phase by (-i)^{popcount(x & z) mod 4}; real when possible.

        ``device`` (not in the reference): a CUDA device on which the consolidation, grouping
        and phasing run (``rq_terms_group``); the labels are parsed into X / Z masks on the host.
        The result is the same, bit for bit."""
        if device is not None and isinstance(paulisum, tuple):
            return cls._from_paulisum_device(paulisum, force_real, add_padding, device)
        if isinstance(paulisum, tuple):
            paulis, coeffs = paulisum
            if len(paulis) != len(coeffs):
                raise ValueError('Lengths of Pauli and coeff lists do not match')
            if len(set(len(p) for p in paulis)) != 1:
                raise ValueError('Pauli strings have non-uniform lengths')
            coeffs = np.array(coeffs)
            n = len(paulis[0])
            labels = np.array([p.upper() for p in paulis], dtype=f'<U{max(n, 1)}')
            keep = np.nonzero(coeffs)
            coeffs = coeffs[keep]
            labels = labels[keep]
            uniq, inv = np.unique(labels, return_inverse=True)
            summed = np.zeros(len(uniq), dtype=coeffs.dtype)
            np.add.at(summed, inv.ravel(), coeffs)
            coeffs = summed
            codes = uniq.view(np.uint32).reshape(len(uniq), n) if n else np.zeros((len(uniq), 0))
            xbits = (codes == ord('X')) | (codes == ord('Y'))
            zbits = (codes == ord('Y')) | (codes == ord('Z'))
        elif _is_sparse_pauli_op(paulisum):
            if not np.allclose(paulisum.coeffs.imag, 0.):
                raise ValueError('Coefficients of Paulis must be real for the Hamiltonian to be'
                                 ' Hermitian.')
            paulisum = paulisum.simplify()
            coeffs = paulisum.coeffs
            xbits = paulisum.paulis.x[:, ::-1]
            zbits = paulisum.paulis.z[:, ::-1]
            n = paulisum.num_qubits
        else:
            raise ValueError('Unsupported input type')

        if force_real:
            if np.any(np.imag(coeffs) != 0.):
                warnings.warn('Found nonzero imaginary part when force_real=True')
            coeffs = np.real(coeffs)

        xm = bits_to_masks(xbits)
        zm = bits_to_masks(zbits)
        xuniq, indices = np.unique(xm, return_inverse=True)
        indices = indices.ravel()
        order = np.argsort(indices, kind='stable')  # group members keep the string order
        counts = np.bincount(indices, minlength=len(xuniq))
        toff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        zsig = zm[order]
        iph = (np.bitwise_count(xm[order] & zsig) & 3).astype(np.int64)
        phc = np.asarray(coeffs)[order] * _PHASES[iph]
        if np.all(phc.imag == 0.):
            phc = phc.real.copy()
        return cls._from_compact(xuniq, toff, zsig, phc, n, add_padding)

    @classmethod
    def _from_paulisum_device(cls, paulisum, force_real, add_padding, device):
        """The (labels, coeffs) form of from_paulisum with rq_terms_group doing the array work."""
        import ctypes
        import torch
        from .. import _lib as L
        paulis, coeffs = paulisum
        if len(paulis) != len(coeffs):
            raise ValueError('Lengths of Pauli and coeff lists do not match')
        if len(set(len(p) for p in paulis)) != 1:
            raise ValueError('Pauli strings have non-uniform lengths')
        n = len(paulis[0])
        if n > 64:
            raise ValueError('at most 64 qubits are supported')
        labels = np.array([p.upper() for p in paulis], dtype=f'<U{max(n, 1)}')
        codes = labels.view(np.uint32).reshape(len(labels), n) if n else np.zeros((len(labels), 0))
        xm = bits_to_masks((codes == ord('X')) | (codes == ord('Y')))
        zm = bits_to_masks((codes == ord('Y')) | (codes == ord('Z')))
        c_in = np.array(coeffs)
        K = len(labels)
        dev = torch.device(device)

        def u64(a):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).to(dev)

        cin = torch.from_numpy(np.ascontiguousarray(c_in, dtype=np.complex128)).to(dev)
        d_x, d_z = u64(xm), u64(zm)
        xo = torch.empty(K, dtype=torch.int64, device=dev)
        to = torch.empty(K + 1, dtype=torch.int64, device=dev)
        zo = torch.empty(K, dtype=torch.int64, device=dev)
        co = torch.empty(K, dtype=torch.complex128, device=dev)
        nb = ctypes.c_size_t()
        L.check(L.lib().rq_terms_group_scratch_size(K, ctypes.byref(nb)), 'rq_terms_group')
        scratch = torch.empty(int(nb.value), dtype=torch.uint8, device=dev)
        J, K2, flags = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        with torch.cuda.device(dev):
            L.check(L.lib().rq_terms_group(K, L.ptr(d_x), L.ptr(d_z), L.ptr(cin),
                                           int(bool(force_real)), L.ptr(xo), L.ptr(to), L.ptr(zo),
                                           L.ptr(co), ctypes.byref(J), ctypes.byref(K2),
                                           ctypes.byref(flags), L.ptr(scratch), L.stream_ptr()),
                    'rq_terms_group')
        J, K2 = J.value, K2.value
        if flags.value & 1:
            warnings.warn('Found nonzero imaginary part when force_real=True')
        coef = co[:K2].cpu().numpy()
        if flags.value & 2:
            coef = coef.real.copy()
        return cls._from_compact(xo[:J].cpu().numpy().view(np.uint64),
                                 to[:J + 1].cpu().numpy(), zo[:K2].cpu().numpy().view(np.uint64),
                                 coef, n, add_padding)

    # ------------------------------------------------------------------------------------------
    @property
    def num_groups(self):
        return len(self.xmask)

    @property
    def is_real(self):
        return not np.iscomplexobj(self.coef)

    def _packed_arrays(self):
        if self._packed is None:
            n, J = self.num_qubits, len(self.xmask)
            counts = np.diff(self.toff)
            kmax = int(counts.max()) if J else 0
            zfull = np.zeros((J, kmax), dtype=np.uint64)
            cfull = np.zeros((J, kmax), dtype=self.coef.dtype)
            for j in range(J):
                a, b = self.toff[j], self.toff[j + 1]
                zfull[j, :b - a] = self.zmask[a:b]
                cfull[j, :b - a] = self.coef[a:b]
            self._packed = (masks_to_packed(self.xmask, n, self.padded),
                            masks_to_packed(zfull, n, self.padded), cfull)
        return self._packed

    @property
    def x(self):
        return self._packed_arrays()[0]

    @property
    def z(self):
        return self._packed_arrays()[1]

    @property
    def c(self):
        return self._packed_arrays()[2]

    @property
    def arrays(self):
        """(x, z, c) in the reference's packed layout (symplectic.py:127-129)."""
        return self._packed_arrays()

    def device_arrays(self, truncate=True):
        """Host arrays of the C ABI's grouped terms: (xmask, toff int32, zmask, coef complex128,
        diag_group, is_real).  With ``truncate`` each group ends at its first zero coefficient,
        the reference's diagonal loop (sqd.py:561-575); without, every term is kept
        (PauliSumXZ.matmul, symplectic.py:142-147)."""
        J = len(self.xmask)
        coef = self.coef.astype(np.complex128)
        keep = np.ones(len(coef), dtype=bool)
        if truncate:
            zero = coef == 0
            for j in range(J):
                a, b = int(self.toff[j]), int(self.toff[j + 1])
                zs = np.nonzero(zero[a:b])[0]
                if len(zs):
                    keep[a + zs[0]:b] = False
        counts = np.array([int(keep[self.toff[j]:self.toff[j + 1]].sum()) for j in range(J)],
                          dtype=np.int64) if J else np.zeros(0, np.int64)
        toff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        diag = np.nonzero(self.xmask == 0)[0]
        diag_group = int(diag[0]) if len(diag) else -1
        return (self.xmask.copy(), toff, self.zmask[keep].copy(), coef[keep].copy(), diag_group,
                bool(np.all(coef.imag == 0)))

    # ------------------------------------------------------------------------------------------
    def matmul(self, rhs):
        """Full-space product H @ rhs with rhs of shape (2^n,) or (2^n, m) (symplectic.py:131-150),
        on the GPU.  Returns the type of ``rhs`` (NumPy in, NumPy out; torch in, torch out)."""
        from ..device import fullspace_matmul
        if rhs.shape[0] != 2 ** self.num_qubits:
            raise ValueError(f'RHS axis 0 size {rhs.shape[0]} is incompatible with'
                             f' num_qubits={self.num_qubits}')
        return fullspace_matmul(self, rhs)

    def __repr__(self):
        return (f'PauliSumXZ(num_qubits={self.num_qubits}, groups={len(self.xmask)}, '
                f'terms={len(self.zmask)}, dtype={self.coef.dtype})')


def _trimmed_len(row):
    """Number of entries of a padded coefficient row up to its last nonzero one."""
    nz = np.nonzero(np.asarray(row))[0]
    return int(nz[-1]) + 1 if len(nz) else 0
