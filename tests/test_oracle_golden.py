"""The CPU oracle against fixtures recorded from the reference's own code (CPU only)."""
import warnings

import numpy as np
import pytest

from golden_cases import case_names, load, packed_to_u64, hamiltonian
from oracle import paulis as opaulis, sqd as osqd, dense as odense
from oracle.ground_locg import ground_locg, eigenpair_3x3, eigenpair_2x2

CASES = case_names()


def _terms(case, force_real=True):
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        return opaulis.from_paulisum(hamiltonian(case), force_real=force_real)


@pytest.mark.parametrize('name', CASES)
def test_from_paulisum_matches_reference(name):
    case = load(name)
    t = _terms(case)
    x, z = t.to_reference_packed(add_padding=True)
    np.testing.assert_array_equal(x, case['ham_x'])
    np.testing.assert_array_equal(z, case['ham_z'])
    assert t.c.dtype == case['ham_c'].dtype
    np.testing.assert_allclose(t.c, case['ham_c'], rtol=0, atol=1e-15)
    t2 = _terms(case, force_real=False)
    x2, z2 = t2.to_reference_packed(add_padding=False)
    np.testing.assert_array_equal(x2, case['nopad_x'])
    np.testing.assert_array_equal(z2, case['nopad_z'])
    np.testing.assert_allclose(t2.c, case['nopad_c'], rtol=0, atol=1e-15)


@pytest.mark.parametrize('name', CASES)
def test_subspace_and_connectivity_bit_exact(name):
    case = load(name)
    n, D = int(case['num_qubits']), int(case['D'])
    S = osqd.uniquify(osqd.pack_states(case['states']))
    np.testing.assert_array_equal(S, packed_to_u64(case['states_u'][:D], n))
    t = _terms(case)
    ref = case['xsources'][:, :D]
    np.testing.assert_array_equal(osqd.xsources_all(S, t), ref)
    for j, xv in enumerate(t.x):
        np.testing.assert_array_equal(osqd.xsource_search(S, xv), ref[j])


@pytest.mark.parametrize('name', CASES)
def test_diagonals_matvec_vinit(name):
    case = load(name)
    D = int(case['D'])
    t = _terms(case)
    S = osqd.uniquify(osqd.pack_states(case['states']))
    for j in range(len(t.x)):
        np.testing.assert_allclose(osqd.diagonal(S, t.z[j], t.c[j]), case['diagonals'][j, :D],
                                   rtol=1e-13, atol=1e-13)
    xs = osqd.xsources_all(S, t)
    for v, out in zip(case['mv_in'], case['mv_out']):
        got = osqd.matvec_xcached(v[:D], xs, t, S)
        np.testing.assert_allclose(got, out[:D], rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(osqd.initial_vector(t, S), case['vinit'][:D])


def test_zero_coefficient_truncates_group():
    """A consolidated coefficient of exactly 0 stops its group's diagonal loop (sqd.py:562-564)."""
    case = load('zero_coeff')
    t = _terms(case)
    zero_groups = [j for j in range(len(t.x)) if np.any(t.c[j, :t.counts[j]] == 0)]
    assert zero_groups, 'fixture must contain a group with a zero coefficient'
    S = osqd.uniquify(osqd.pack_states(case['states']))
    j = zero_groups[0]
    first0 = int(np.nonzero(t.c[j] == 0)[0][0])
    full = np.zeros(len(S), dtype=t.c.dtype)
    for zk, ck in zip(t.z[j][:t.counts[j]], t.c[j][:t.counts[j]]):
        full = full + ck * (1 - 2 * osqd.popparity(S & np.uint64(zk)))
    trunc = osqd.diagonal(S, t.z[j], t.c[j])
    if first0 < t.counts[j] - 1:
        assert not np.allclose(full, trunc)
    np.testing.assert_allclose(trunc, case['diagonals'][j, :int(case['D'])], atol=1e-14)
    # the reference's eigenvalue is that of the truncated operator, not of the full sum
    w_trunc = np.linalg.eigvalsh(osqd.hproj_dense(t, S))[0]
    w_full = odense.projected_ground(*hamiltonian(case), S)[0]
    assert abs(float(case['eigval']) - w_trunc) < 1e-9
    assert abs(w_full - w_trunc) > 1e-6


@pytest.mark.parametrize('name', CASES)
def test_lobpcg_matches_reference(name):
    case = load(name)
    D = int(case['D'])
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        eig, vec, basis, niter = osqd.sqd(hamiltonian(case), case['states'],
                                          states_size=int(case['states_size']))
    assert niter == int(case['niter'])
    ref = float(case['eigval'])
    if np.isnan(ref):
        assert np.isnan(eig)
        return
    assert abs(eig - ref) <= 1e-10 * max(1., abs(ref))
    np.testing.assert_allclose(vec, case['eigvec'], rtol=0, atol=1e-8)
    np.testing.assert_array_equal(basis, case['basis'])
    assert vec.shape == (D,)


@pytest.mark.parametrize('name', [n for n in CASES if n not in ('local20', 'n16', 'zero_coeff')])
def test_dense_eigh_acceptance(name):
    """tests/sqd.ipynb cell 3 restated: eigenvalue equals eigh of the projected dense matrix."""
    case = load(name)
    S = osqd.uniquify(osqd.pack_states(case['states']))
    p, c = hamiltonian(case)
    t = _terms(case)
    if int(case['num_qubits']) > 12:
        # 2^n x 2^n is too large: eigh of the projected matrix built from the grouped form
        w, v = np.linalg.eigh(osqd.hproj_dense(t, S))
        assert abs(float(case['eigval']) - w[0]) <= 1e-8 * max(1., abs(w[0]))
        assert abs(np.vdot(v[:, 0], case['eigvec'])) > 1 - 1e-6
        return
    w0, v0, Hp = odense.projected_ground(p, c, S)
    assert abs(float(case['eigval']) - w0) <= 1e-8 * max(1., abs(w0))
    assert abs(np.vdot(v0, case['eigvec'])) > 1 - 1e-6
    # the grouped (symplectic) matrix equals the Kronecker-product matrix element-wise
    np.testing.assert_allclose(osqd.hproj_dense(t, S), Hp, atol=1e-12)


def test_fullspace_matmul():
    case = load('fullspace')
    t = opaulis.from_reference_arrays(case['ham_x'], case['ham_z'], case['ham_c'],
                                      int(case['num_qubits']), padded=False)
    np.testing.assert_allclose(odense.fullspace_matmul(t, case['rhs1']), case['out1'], atol=1e-12)
    H = odense.hamiltonian_matrix([str(p) for p in case['paulis']], case['coeffs'])
    np.testing.assert_allclose(H @ case['rhs1'], case['out1'], atol=1e-12)


def test_sortmerge_equals_search_random():
    rng = np.random.default_rng(3)
    S = np.unique(rng.integers(0, 1 << 40, size=5000, dtype=np.uint64))
    for _ in range(20):
        x = np.uint64(rng.integers(0, 1 << 40))
        np.testing.assert_array_equal(osqd.xsource_sortmerge(S, x), osqd.xsource_search(S, x))
    # x = 0 maps every row to itself
    np.testing.assert_array_equal(osqd.xsource_sortmerge(S, 0), np.arange(len(S)))


def test_small_eigenpairs():
    rng = np.random.default_rng(5)
    for _ in range(50):
        a = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        h = a + a.conj().T
        lam, v = eigenpair_3x3(h)
        w = np.linalg.eigvalsh(h)
        assert abs(lam - w[0]) < 1e-10
        np.testing.assert_allclose(h @ v, lam * v, atol=1e-9)
        b = h[:2, :2]
        lam2, v2 = eigenpair_2x2(b)
        assert abs(lam2 - np.linalg.eigvalsh(b)[0]) < 1e-10


def test_ground_locg_integer_xinit_and_matrix():
    rng = np.random.default_rng(9)
    a = rng.normal(size=(40, 40))
    h = a + a.T
    theta, x, niter = ground_locg(lambda v: h @ v, 0, vspace=(40, np.float64))
    assert abs(theta - np.linalg.eigvalsh(h)[0]) < 1e-10
