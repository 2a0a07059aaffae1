"""Host-side logic of the package against the reference fixtures (CPU only)."""
import warnings

import numpy as np
import pytest

from golden_cases import case_names, load, hamiltonian, packed_to_u64
from rqutils_gb300.paulis.symplectic import PauliSumXZ
from rqutils_gb300 import sqd as psqd
from rqutils_gb300 import workloads

CASES = case_names()


@pytest.mark.parametrize('name', CASES)
def test_from_paulisum_packed_matches_reference(name):
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        h = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True, add_padding=True)
        h2 = PauliSumXZ.from_paulisum(hamiltonian(case))
    np.testing.assert_array_equal(h.x, case['ham_x'])
    np.testing.assert_array_equal(h.z, case['ham_z'])
    assert h.c.dtype == case['ham_c'].dtype
    np.testing.assert_allclose(h.c, case['ham_c'], atol=1e-15, rtol=0)
    np.testing.assert_array_equal(h2.x, case['nopad_x'])
    np.testing.assert_array_equal(h2.z, case['nopad_z'])
    np.testing.assert_allclose(h2.c, case['nopad_c'], atol=1e-15, rtol=0)
    # round trip through the reference's packed constructor
    h3 = PauliSumXZ(case['ham_x'], case['ham_z'], case['ham_c'], int(case['num_qubits']))
    assert h3.padded
    np.testing.assert_array_equal(h3.xmask, h.xmask)


def test_from_paulisum_errors():
    with pytest.raises(ValueError, match='Lengths'):
        PauliSumXZ.from_paulisum((['XX', 'YY'], [1.]))
    with pytest.raises(ValueError, match='non-uniform'):
        PauliSumXZ.from_paulisum((['XX', 'YYY'], [1., 2.]))
    with pytest.raises(ValueError, match='Unsupported'):
        PauliSumXZ.from_paulisum([('XX', 1.)])
    with pytest.warns(UserWarning, match='imaginary'):
        PauliSumXZ.from_paulisum((['XX', 'ZZ'], [1., 1j]), force_real=True)


def test_truncation_at_first_zero():
    # 'XXII' (+0.5 - 0.5 = 0) precedes 'XXZI' and 'YYII' in its group: both are dropped
    h = PauliSumXZ.from_paulisum((['XXII', 'XXII', 'XXZI', 'YYII', 'ZIII'],
                                  [0.5, -0.5, 0.7, -0.3, 1.0]), force_real=True)
    xm, toff, zm, cf, dg, real = h.device_arrays(truncate=True)
    g = int(np.nonzero(xm == 0b1100)[0][0])
    assert toff[g + 1] - toff[g] == 0
    xm2, toff2, *_ = h.device_arrays(truncate=False)
    assert toff2[g + 1] - toff2[g] == 3


@pytest.mark.parametrize('name', CASES)
def test_subspace_states(name):
    case = load(name)
    n, D = int(case['num_qubits']), int(case['D'])
    S = psqd.subspace_states(case['states'], n)
    np.testing.assert_array_equal(S, packed_to_u64(case['states_u'][:D], n))
    np.testing.assert_array_equal(psqd.unpack_states(S, n), case['basis'])
    assert np.array_equal(psqd.subspace_states(S, n), S)
    with pytest.raises(ValueError, match='strictly increasing'):
        psqd.subspace_states(S[::-1].copy(), n)


def test_cache_modes():
    assert psqd.cache_mode((1, 0)) == 'conn'
    assert psqd.cache_mode((0, 0)) == 'free'
    assert psqd.cache_mode((1, 2)) == 'csr'
    assert psqd.cache_mode((0, 1)) == 'free'
    with pytest.raises(ValueError):
        psqd.cache_mode((2, 0))


def test_workload_generators():
    rng = np.random.default_rng(0)
    p, c = workloads.random_pauli_sum(rng, 20, 200)
    assert len(p) == 200 and all(len(s) == 20 for s in p)
    assert all(1 <= sum(ch != 'I' for ch in s) <= 4 for s in p)
    hp, hc = workloads.hubbard_jw(4, 4, 1.0, 4.0)
    h = PauliSumXZ.from_paulisum((hp, hc), force_real=True)
    assert h.num_qubits == 32 and h.is_real
    assert len(h.xmask) == 65 and len(h.zmask) == 177
    S = workloads.sample_sector(rng, 5000, [(16, 8), (16, 8)])
    assert len(S) == 5000 and np.all(S[1:] > S[:-1])
    lo = S & np.uint64(0xFFFF)
    assert np.all(np.bitwise_count(lo) == 8) and np.all(np.bitwise_count(S >> np.uint64(16)) == 8)
    S2 = workloads.sample_sector(rng, 100000, [(20, 10)])
    assert np.all(np.bitwise_count(S2) == 10) and len(np.unique(S2)) == 100000


def test_hubbard_matches_dense_small():
    """Our JW Hubbard mapping has the exact 2x2 spectrum at half filling (sector energies)."""
    from oracle import dense
    p, c = workloads.hubbard_jw(2, 1, 1.0, 4.0, periodic=False)
    H = dense.hamiltonian_matrix(p, c)
    # two sites, one up and one down electron: E0 = (U - sqrt(U^2 + 16 t^2)) / 2
    idx = [i for i in range(16) if bin(i & 0b11).count('1') == 1 and bin(i >> 2).count('1') == 1]
    w = np.linalg.eigvalsh(H[np.ix_(idx, idx)])
    assert abs(w[0] - (4 - np.sqrt(16 + 16)) / 2) < 1e-12


def _jw_matrices(n):
    """a_p as explicit matrices: Z on qubits below p, |0><1| on p (character 0 = qubit n-1)."""
    I2, Z = np.eye(2), np.diag([1., -1.])
    lower = np.array([[0, 1], [0, 0]], dtype=complex)
    ops = []
    for p in range(n):
        m = np.ones((1, 1))
        for q in range(n - 1, -1, -1):
            m = np.kron(m, Z if q < p else (lower if q == p else I2))
        ops.append(m)
    return ops


@pytest.mark.parametrize('ns', [1, 2, 3])
def test_chemistry_jw_matches_fermion_matrices(ns):
    """The vectorised Jordan-Wigner mapping equals the second-quantised operator built from
    explicit ladder matrices."""
    from oracle import dense
    labels, coeffs = workloads.chemistry_jw(ns, np.random.default_rng(5))
    H = dense.hamiltonian_matrix(labels, coeffs)
    rng = np.random.default_rng(5)
    h = rng.normal(0, 1 / np.sqrt(ns), size=(ns, ns))
    h = 0.5 * (h + h.T)
    g = workloads._random_eri(rng, ns, 0.1)
    n = 2 * ns
    a = _jw_matrices(n)
    ad = [m.conj().T for m in a]
    ref = np.zeros((2 ** n,) * 2, dtype=complex)
    for s in (0, ns):
        for p in range(ns):
            for q in range(ns):
                ref += h[p, q] * ad[p + s] @ a[q + s]
    for s in (0, ns):
        for t in (0, ns):
            for p in range(ns):
                for q in range(ns):
                    for r in range(ns):
                        for u in range(ns):
                            ref += 0.5 * g[p, q, r, u] * ad[p + s] @ ad[r + t] @ a[u + t] @ a[q + s]
    np.testing.assert_allclose(H, ref, atol=1e-13)


def test_chemistry_truncation_keeps_largest():
    labels, coeffs = workloads.chemistry_jw(4, np.random.default_rng(1), keep=50)
    full_l, full_c = workloads.chemistry_jw(4, np.random.default_rng(1))
    assert len(labels) == 50
    assert np.min(np.abs(coeffs)) >= np.sort(np.abs(full_c))[-50] - 1e-15


def test_batch_composite_keys_and_terms():
    """Host layout of a batch: composite keys sorted by (problem, state), row and group ranges
    consistent with each problem's own grouped terms."""
    from rqutils_gb300.batch import STATE_BITS, composite_keys, concat_terms
    hams_raw, states, ns = workloads.batched_random_problems(3, P=6, d_range=(16, 300),
                                                             k_range=(10, 60))
    hams = [PauliSumXZ.from_paulisum(h, force_real=True, add_padding=True) for h in hams_raw]
    keys, prow = composite_keys(states)
    assert np.all(keys[1:] > keys[:-1])
    assert prow[0] == 0 and prow[-1] == len(keys)
    for p, s in enumerate(states):
        seg = keys[prow[p]:prow[p + 1]]
        assert np.all((seg >> np.uint64(STATE_BITS)) == p)
        np.testing.assert_array_equal(seg & np.uint64((1 << STATE_BITS) - 1), s)
    xm, toff, zm, cf, gofs, dgrp, real = concat_terms(hams)
    for p, h in enumerate(hams):
        x1, t1, z1, c1, dg1, _ = h.device_arrays(truncate=True)
        g0, g1 = gofs[p], gofs[p + 1]
        np.testing.assert_array_equal(xm[g0:g1], x1)
        np.testing.assert_array_equal(toff[g0:g1 + 1] - toff[g0], t1)
        np.testing.assert_array_equal(zm[toff[g0]:toff[g1]], z1)
        np.testing.assert_array_equal(cf[toff[g0]:toff[g1]], c1)
        assert dgrp[p] == (g0 + dg1 if dg1 >= 0 else -1)
    with pytest.raises(ValueError):
        composite_keys([np.array([1 << STATE_BITS], np.uint64)])


def test_batched_random_problems_shapes():
    hams, states, ns = workloads.batched_random_problems(4, P=12, d_range=(2 ** 6, 2 ** 10),
                                                         k_range=(100, 200))
    for (lab, c), s, n in zip(hams, states, ns):
        assert 16 <= n <= 40 and len(lab[0]) == n
        assert 100 <= len(lab) <= 200
        assert np.all(s[1:] > s[:-1])
        assert np.all(np.bitwise_count(s) == n // 2)
        assert 1 <= len(s) <= 2 ** 10
