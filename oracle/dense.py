"""Independent dense checks -- test infrastructure only.

* ``pauli_matrix`` / ``hamiltonian_matrix`` build H from Kronecker products of 2x2 Pauli matrices
  (no symplectic form involved), the same check the reference's only SQD test performs with
  ``SparsePauliOp.to_matrix()`` (``tests/sqd.ipynb`` cell 3).
* ``projected_ground`` restates that notebook's acceptance test: rows/columns of H at the sorted
  unique states, then ``eigh``.
* ``fullspace_matmul`` restates ``PauliSumXZ.matmul`` (``rqutils/paulis/symplectic.py:131-150``):
  the same row-side formula with the identity projection, D = 2^n.
"""
import numpy as np

from .paulis import OracleTerms
from .sqd import popparity

_SIGMA = {
    'I': np.eye(2, dtype=np.complex128),
    'X': np.array([[0, 1], [1, 0]], dtype=np.complex128),
    'Y': np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    'Z': np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def pauli_matrix(label):
    """Kronecker product with character 0 as the most significant qubit (qubit n-1)."""
    m = np.ones((1, 1), dtype=np.complex128)
    for ch in label.upper():
        m = np.kron(m, _SIGMA[ch])
    return m


def hamiltonian_matrix(paulis, coeffs):
    n = len(paulis[0])
    H = np.zeros((2 ** n, 2 ** n), dtype=np.complex128)
    for p, c in zip(paulis, coeffs):
        H += c * pauli_matrix(p)
    return H


def projected_ground(paulis, coeffs, states_u64, force_real=True):
    """Lowest eigenpair of H restricted to the given sorted basis states (tests/sqd.ipynb cell 3).
    With ``force_real`` the coefficients are cast to real first, as ``sqd()`` does."""
    coeffs = np.asarray(coeffs)
    if force_real:
        coeffs = np.real(coeffs)
    H = hamiltonian_matrix(paulis, coeffs)
    idx = np.asarray(states_u64, dtype=np.int64)
    w, v = np.linalg.eigh(H[np.ix_(idx, idx)])
    return w[0], v[:, 0], H[np.ix_(idx, idx)]


def fullspace_matmul(terms: OracleTerms, rhs):
    """PauliSumXZ.matmul (symplectic.py:131-150): out[i] = sum_j rhs[i ^ x_j] sum_k c_jk
    (1 - 2 parity(i & z_jk)) over every stored coefficient (padding contributes zero)."""
    n = terms.num_qubits
    if rhs.shape[0] != 2 ** n:
        raise ValueError(f'RHS axis 0 size {rhs.shape[0]} is incompatible with num_qubits={n}')
    idx = np.arange(2 ** n, dtype=np.uint64)
    out = np.zeros(rhs.shape, dtype=np.result_type(rhs.dtype, terms.c.dtype))
    for j in range(len(terms.x)):
        diag = np.zeros(2 ** n, dtype=terms.c.dtype)
        for zk, ck in zip(terms.z[j], terms.c[j]):
            diag = diag + ck * (1. - 2. * popparity(idx & np.uint64(zk)))
        src = (idx ^ np.uint64(terms.x[j])).astype(np.int64)
        out = out + rhs[src] * diag.reshape((-1,) + (1,) * (rhs.ndim - 1))
    return out
