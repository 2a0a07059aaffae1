"""CUDA path against the reference fixtures and the oracle (GPU)."""
import warnings

import numpy as np
import pytest

from golden_cases import case_names, load, hamiltonian

pytestmark = pytest.mark.gpu

CASES = case_names()
CONVERGING = [c for c in CASES if c not in ('local20', 'n16')]


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _problem(case, cache_level=(1, 0), lookup='hash'):
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import SQDProblem, subspace_states
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        h = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True, add_padding=True)
    S = subspace_states(case['states'], h.num_qubits)
    return SQDProblem(h, S, cache_level=cache_level, lookup=lookup), h, S


@pytest.mark.parametrize('lookup', ['hash', 'bsearch'])
@pytest.mark.parametrize('name', CASES)
def test_xsource_bit_exact(name, lookup):
    case = load(name)
    prob, h, S = _problem(case, cache_level=(0, 0), lookup=lookup)
    D = int(case['D'])
    got = prob.sub.xsource(h.xmask).cpu().numpy()
    np.testing.assert_array_equal(got, case['xsources'][:, :D])


@pytest.mark.parametrize('name', CASES)
def test_group_diagonals(name):
    case = load(name)
    prob, h, S = _problem(case, cache_level=(0, 0))
    D = int(case['D'])
    for j in range(len(h.xmask)):
        d = prob.op.group_diagonal(j).cpu().numpy()
        ref = case['diagonals'][j, :D]
        np.testing.assert_allclose(d if np.iscomplexobj(ref) else d.real, ref, rtol=1e-13,
                                   atol=1e-13)


@pytest.mark.parametrize('mode', [(0, 0), (1, 0), (1, 2)])
@pytest.mark.parametrize('name', CASES)
def test_matvec_fp64(name, mode):
    import torch
    case = load(name)
    prob, h, S = _problem(case, cache_level=mode)
    D = int(case['D'])
    for v, ref in zip(case['mv_in'], case['mv_out']):
        x = torch.as_tensor(v[:D]).cuda()
        y = prob.op.matvec(x).cpu().numpy()
        np.testing.assert_allclose(y, ref[:D], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize('name', CASES)
def test_matvec_fp32_error_bound(name):
    """complex64 / float32 matvec: relative error <= 1e-6 against the FP64 reference output."""
    import torch
    case = load(name)
    for mode in [(0, 0), (1, 0)]:
        prob, h, S = _problem(case, cache_level=mode)
        D = int(case['D'])
        for v, ref in zip(case['mv_in'], case['mv_out']):
            dt = torch.float32 if h.is_real else torch.complex64
            x = torch.as_tensor(v[:D]).to(dt).cuda()
            y = prob.op.matvec(x).cpu().numpy().astype(ref.dtype)
            # error of the 32-bit product relative to the exact product of the rounded input
            exact = prob.op.matvec(x.to(torch.float64 if h.is_real else torch.complex128))
            e = np.linalg.norm(y - exact.cpu().numpy()) / np.linalg.norm(exact.cpu().numpy())
            assert e <= 1e-6, e
            e2 = np.linalg.norm(y - ref[:D]) / np.linalg.norm(ref[:D])
            assert e2 <= 1e-6, e2


@pytest.mark.parametrize('name', CASES)
def test_connectivity_matches_reference_table(name):
    case = load(name)
    prob, h, S = _problem(case, cache_level=(1, 0))
    D = int(case['D'])
    rowptr, col, grp = prob.op.connectivity()
    xs = case['xsources'][:, :D]
    dg = prob.terms.diag_group
    exp_col, exp_grp, exp_ptr = [], [], [0]
    for i in range(D):
        for j in range(xs.shape[0]):
            if j != dg and xs[j, i] >= 0:
                exp_col.append(xs[j, i])
                exp_grp.append(j)
        exp_ptr.append(len(exp_col))
    np.testing.assert_array_equal(rowptr, exp_ptr)
    np.testing.assert_array_equal(col, exp_col)
    np.testing.assert_array_equal(grp, exp_grp)


@pytest.mark.parametrize('name', CASES)
def test_sqd_matches_reference(name):
    from rqutils_gb300.sqd import sqd
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        eig, vec, basis, info = sqd(hamiltonian(case), case['states'],
                                    states_size=int(case['states_size']), return_info=True)
    ref = float(case['eigval'])
    np.testing.assert_array_equal(basis, case['basis'])
    if np.isnan(ref):
        assert np.isnan(eig) and info['niter'] == int(case['niter'])
        return
    assert abs(eig - ref) <= 1e-10 * max(1., abs(ref)), (eig, ref)
    assert abs(np.vdot(case['eigvec'], vec)) > 1 - 1e-9
    assert vec.dtype == case['eigvec'].dtype
    # same algorithm and operation order up to reduction order: iteration counts agree closely
    assert abs(info['niter'] - int(case['niter'])) <= max(2, int(0.05 * int(case['niter'])))


@pytest.mark.parametrize('name', CONVERGING)
@pytest.mark.parametrize('variant', ['reference', 'fast'])
@pytest.mark.parametrize('cache_level', [(0, 0), (1, 2)])
def test_sqd_modes_and_variants(name, variant, cache_level):
    from rqutils_gb300.sqd import sqd
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        eig = sqd(hamiltonian(case), case['states'], return_eigvec=False, variant=variant,
                  cache_level=cache_level)
    ref = float(case['eigval'])
    assert abs(eig - ref) <= 1e-9 * max(1., abs(ref)), (eig, ref)


@pytest.mark.parametrize('name', ['notebook', 'hubbard2x2', 'local12', 'n16dense'])
def test_sqd_mixed_precision(name):
    from rqutils_gb300.sqd import sqd
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        eig, vec, _, info = sqd(hamiltonian(case), case['states'], precision='mixed',
                                return_info=True)
    ref = float(case['eigval'])
    assert abs(eig - ref) <= 1e-8 * max(1., abs(ref)), (eig, ref, info)


def test_fullspace_matmul():
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    case = load('fullspace')
    h = PauliSumXZ.from_paulisum(([str(p) for p in case['paulis']], case['coeffs']))
    out = h.matmul(case['rhs1'])
    np.testing.assert_allclose(out, case['out1'], rtol=1e-12, atol=1e-12)
    two = h.matmul(np.stack([case['rhs1'], 2 * case['rhs1']], axis=1))
    np.testing.assert_allclose(two[:, 1], 2 * case['out1'], rtol=1e-12, atol=1e-12)


def test_ground_locg_callable_and_matrix():
    import torch
    from rqutils_gb300.ground_locg import ground_locg
    from oracle.ground_locg import ground_locg as oracle_locg
    rng = np.random.default_rng(4)
    a = rng.normal(size=(60, 60)) + 1j * rng.normal(size=(60, 60))
    h = a + a.conj().T
    x0 = np.zeros(60, complex)
    x0[3] = 1
    th_o, x_o, n_o = oracle_locg(lambda v: h @ v, x0)
    th, x, n = ground_locg(h, x0)
    assert abs(th - np.linalg.eigvalsh(h)[0]) < 1e-10
    assert abs(th - th_o) < 1e-10 and abs(n - n_o) <= 2
    ht = torch.as_tensor(h).cuda()
    th2, x2, n2 = ground_locg(lambda v, s: s * (ht @ v), 3, args=(1.0,), vspace=(60, np.complex128))
    assert abs(th2 - th) < 1e-10 and isinstance(x2, np.ndarray)


def test_unsorted_subspace_rejected():
    from rqutils_gb300.device import DeviceSubspace
    from rqutils_gb300._lib import RqError
    with pytest.raises(RqError, match='strictly increasing'):
        DeviceSubspace(np.array([1, 5, 3], dtype=np.uint64), num_qubits=4)
    with pytest.raises(RqError):
        DeviceSubspace(np.array([1, 5, 5], dtype=np.uint64), num_qubits=4)


def test_extreme_keys_and_empty_choice():
    """States containing both 0 and 2^64-1 force the empty key into a gap."""
    import torch
    from rqutils_gb300.device import DeviceSubspace
    S = np.array([0, 1, 2, 7, 2 ** 63, 2 ** 64 - 2, 2 ** 64 - 1], dtype=np.uint64)
    sub = DeviceSubspace(S, num_qubits=64, filter_masks=(0, 0))
    assert sub.c.empty_key == 3
    xs = sub.xsource(np.array([0, 1, 2 ** 64 - 1, 5], dtype=np.uint64)).cpu().numpy()
    from oracle.sqd import xsource_search
    for j, x in enumerate([0, 1, 2 ** 64 - 1, 5]):
        np.testing.assert_array_equal(xs[j], xsource_search(S, x))


@pytest.mark.parametrize('name', ['notebook', 'local20', 'n16dense'])
def test_key_widths_agree(name):
    """Forced 64-bit keys on problems that also fit 32-bit keys give the same tables."""
    from rqutils_gb300.device import DeviceSubspace
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import subspace_states
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        h = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True)
    S = subspace_states(case['states'], h.num_qubits)
    a = DeviceSubspace(S, num_qubits=h.num_qubits, key_bits=32).xsource(h.xmask).cpu().numpy()
    b = DeviceSubspace(S, num_qubits=h.num_qubits, key_bits=64).xsource(h.xmask).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, case['xsources'][:, :int(case['D'])])


@pytest.fixture(scope='module')
def chem40():
    """40-qubit chemistry-shaped problem (64-bit keys): 20 spatial orbitals, 3000 terms,
    20000 states at 10 alpha + 10 beta electrons."""
    from rqutils_gb300 import workloads
    from oracle.paulis import from_paulisum as oterms
    from oracle import sqd as osqd
    rng = np.random.default_rng(21)
    labels, coeffs = workloads.chemistry_jw(20, rng, keep=3000)
    S = workloads.sample_sector(rng, 20000, [(20, 10), (20, 10)])
    t = oterms((labels, coeffs), force_real=True)
    xs = np.stack([osqd.xsource_search(S, xv) for xv in t.x])
    v = workloads.random_vector(rng, len(S))
    ref = osqd.matvec_xcached(v, xs, t, S)
    return labels, coeffs, S, v, ref, xs


@pytest.mark.parametrize('cache_level', [(0, 0), (1, 0), (1, 2)])
@pytest.mark.parametrize('lookup', ['hash', 'bsearch'])
def test_chemistry_64bit_matvec(chem40, cache_level, lookup):
    import torch
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import SQDProblem
    labels, coeffs, S, v, ref, xs = chem40
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    prob = SQDProblem(h, S, cache_level=cache_level, lookup=lookup)
    assert prob.sub.key_bits == 64
    y = prob.op.matvec(torch.as_tensor(v).cuda()).cpu().numpy()
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    y32 = prob.op.matvec(torch.as_tensor(v).to(torch.complex64).cuda()).cpu().numpy()
    assert np.linalg.norm(y32 - ref) <= 1e-6 * np.linalg.norm(ref)
    got = prob.sub.xsource(h.xmask).cpu().numpy()
    np.testing.assert_array_equal(got, xs)


@pytest.mark.parametrize('mode', ['free', 'conn'])
def test_presence_bitmap_keeps_results(chem40, mode):
    """A presence bitmap forced onto a small table (it is built automatically only for tables
    that do not fit in L2) changes no product and no connectivity list."""
    import torch
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    labels, coeffs, S, v, ref, xs = chem40
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    terms = DeviceTerms(h)
    plain = DeviceSubspace(S, num_qubits=h.num_qubits, presence=False)
    assert plain.pbits == 0
    withp = DeviceSubspace(S, num_qubits=h.num_qubits, presence=plain.hbits + 2)
    assert withp.pbits == plain.hbits + 2
    words = withp.pmap.cpu().numpy().view(np.uint32)
    assert 0 < int(np.bitwise_count(words).sum()) <= len(S)
    x = torch.as_tensor(v).cuda()
    a = DeviceOperator(terms, plain, mode=mode)
    b = DeviceOperator(terms, withp, mode=mode)
    ya, yb = a.matvec(x), b.matvec(x)
    b.check_errors()
    assert torch.equal(ya, yb)
    assert np.linalg.norm(yb.cpu().numpy() - ref) <= 1e-12 * np.linalg.norm(ref)
    if mode == 'conn':
        for u, w in zip(a.connectivity(), b.connectivity()):
            np.testing.assert_array_equal(u, w)


def test_presence_bitmap_and_line_filter_batched():
    """Batched products with a forced presence bitmap and with the line filter (256 to 1024-bit
    lines, each problem with its own prefix shift) equal the product with neither, bit for bit,
    and so do the cached connectivity lists built through them."""
    import torch
    from rqutils_gb300.batch import BatchedSQD
    from rqutils_gb300.workloads import batched_random_problems
    hams, states, ns = batched_random_problems(17, P=6, d_range=(200, 3000), k_range=(50, 200))
    a = BatchedSQD(hams, states, presence=False, line_filter=False)
    b = BatchedSQD(hams, states, presence=int(a.c.hbits) + 2, line_filter=False)
    assert b.pbits > 0
    rng = np.random.default_rng(1)
    x = torch.as_tensor(rng.normal(size=a.D) + 1j * rng.normal(size=a.D)).cuda()
    ya = a.matvec(x)
    assert torch.equal(ya, b.matvec(x))
    b.check_errors()
    for lb in (8, 9, 10):
        c = BatchedSQD(hams, states, line_filter=True, line_bits=lb)
        assert c.lmap is not None and c.pbits == 0
        assert torch.equal(ya, c.matvec(x)), lb
        c.check_errors()
    conn_a = BatchedSQD(hams, states, cache_level=(1, 0), presence=False, line_filter=False)
    conn_c = BatchedSQD(hams, states, cache_level=(1, 0), line_filter=True)
    assert conn_a.nnz == conn_c.nnz
    assert torch.equal(conn_a.col, conn_c.col) and torch.equal(conn_a.grp, conn_c.grp)


@pytest.mark.parametrize('cache_level', [(1, 0), (1, 2)])
@pytest.mark.parametrize('variant', ['reference', 'fast'])
def test_persistent_loop_matches_graph_loop(cache_level, variant):
    """The persistent cooperative kernel (cached-connectivity / CSR operators) and the CUDA-graph
    chunks run the same iteration: same eigenpair, iteration counts within one."""
    import torch
    from rqutils_gb300.ground_locg import lobpcg_solve
    case = load('n16dense')
    prob, h, S = _problem(case, cache_level=cache_level)
    rng = np.random.default_rng(4)
    x0 = torch.as_tensor(rng.normal(size=prob.sub.D)).to(prob.dtype).cuda()
    for mixed in (False, True):
        e1, x1, i1 = lobpcg_solve(prob.op, x0, variant=variant, mixed=mixed, use_graph=1)
        e2, x2, i2 = lobpcg_solve(prob.op, x0, variant=variant, mixed=mixed, use_graph=2)
        assert abs(e1 - e2) <= 1e-12 * abs(e2)
        assert abs(i1['niter'] - i2['niter']) <= 1, (i1, i2)
        assert i1['converged'] and i2['converged']
        assert abs(torch.vdot(x1, x2).item()) > 1 - 1e-10


@pytest.mark.parametrize('use_graph', [1, 2])
def test_fast_restart_converges_to_the_same_eigenpair(use_graph):
    """restart = k (FAST, one problem): the step restarts from x every k iterations of a phase.
    The solve still converges to the eigenpair of the run without restarts, with restarts from
    nearly converged vectors (the restart projects r against x: without that, each restart near
    convergence threw |r| back to ~1e-6 and a 10-iteration period never converged on this
    case); iterations keep counting across restarts, and the reference variant ignores the
    option."""
    import torch
    from rqutils_gb300.ground_locg import lobpcg_solve
    case = load('n16dense')
    prob, h, S = _problem(case, cache_level=(1, 0))
    rng = np.random.default_rng(5)
    x0 = torch.as_tensor(rng.normal(size=prob.sub.D)).to(prob.dtype).cuda()
    for mixed in (False, True):
        e0, x_0, i0 = lobpcg_solve(prob.op, x0, variant='fast', mixed=mixed, use_graph=use_graph)
        e1, x_1, i1 = lobpcg_solve(prob.op, x0, variant='fast', mixed=mixed, use_graph=use_graph,
                                   restart=10)
        assert i0['converged'] and i1['converged'], (i0, i1)
        assert abs(e1 - e0) <= 1e-10 * abs(e0)
        assert abs(torch.vdot(x_0, x_1).item()) > 1 - 1e-8
        if i0['niter'] > 10:
            assert i1['niter'] != i0['niter'] or not torch.equal(x_0, x_1)
        capped = lobpcg_solve(prob.op, x0, variant='fast', mixed=False, use_graph=use_graph,
                              restart=3, maxiter=5)[2]
        assert capped['niter'] == 5 and not capped['converged']
    from rqutils_gb300.sqd import sqd
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        eig = sqd(hamiltonian(case), case['states'], return_eigvec=False, variant='fast',
                  restart=10, use_graph=use_graph)
    assert abs(eig - float(case['eigval'])) <= 1e-9 * abs(float(case['eigval']))
    r0 = lobpcg_solve(prob.op, x0, variant='reference', use_graph=use_graph)
    r1 = lobpcg_solve(prob.op, x0, variant='reference', use_graph=use_graph, restart=10)
    assert r0[0] == r1[0] and r0[2]['niter'] == r1[2]['niter'] and torch.equal(r0[1], r1[1])


@pytest.mark.parametrize('line', [True, False])
@pytest.mark.parametrize('key_bits', [32, 64])
@pytest.mark.parametrize('sectors', ['one', 'two', 'off'])
def test_hash_kernel_sector_filter_modes(sectors, key_bits, line):
    """The FREE hash kernel's three filter forms -- a subspace in one (popcount a, popcount b)
    sector (two popcount compares), several sectors (the bitset) and the filter off -- give the
    oracle's product, and all three agree bit for bit with each other, probing through the line
    filter or the key buckets directly."""
    import torch
    from oracle import sqd as osqd
    from oracle.paulis import from_paulisum as oterms
    from rqutils_gb300 import workloads
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    rng = np.random.default_rng(404)
    n = 16
    labels, coeffs = workloads.random_pauli_sum(rng, n, 300)
    S1 = workloads.sample_sector(rng, 3000, [(8, 4), (8, 4)])
    if sectors == 'two':
        S = np.union1d(S1, workloads.sample_sector(rng, 1500, [(8, 3), (8, 5)]))
    else:
        S = S1
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    ot = oterms((labels, coeffs), force_real=True)
    v = workloads.random_vector(rng, len(S))
    ref = osqd.matvec_xcached(v, osqd.xsources_all(S, ot), ot, S)
    fm = (0, 0) if sectors == 'off' else None
    sub = DeviceSubspace(S, num_qubits=n, filter_masks=fm, key_bits=key_bits, line_filter=line)
    bits = int(np.bitwise_count(sub.fbits.cpu().numpy().view(np.uint32)).sum())
    assert bits == {'one': 1, 'two': 2, 'off': bits}[sectors]
    assert (sub.c.fpoint >= 0) == (sectors == 'one')
    op = DeviceOperator(DeviceTerms(h), sub, mode='free')
    y = op.matvec(torch.as_tensor(v).cuda()).cpu().numpy()
    op.check_errors()
    assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref)
    other = DeviceSubspace(S, num_qubits=n, filter_masks=(0, 0), key_bits=key_bits,
                           line_filter=not line)
    y0 = DeviceOperator(DeviceTerms(h), other, mode='free').matvec(torch.as_tensor(v).cuda()).cpu().numpy()
    np.testing.assert_array_equal(y, y0)


@pytest.mark.parametrize('line_bits', [8, 10])
@pytest.mark.parametrize('key_bits', [32, 64])
@pytest.mark.parametrize('dtype', ['float32', 'float64', 'complex64', 'complex128'])
def test_line_filter_matches_key_buckets(key_bits, dtype, line_bits):
    """2^16 states (buckets with three or four keys and keys moved on from full buckets occur):
    the matrix-free product through the line filter equals, bit for bit, the product through the
    key buckets and the cached-connectivity product; every state sets two bits of one word."""
    import torch
    from rqutils_gb300 import workloads
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    rng = np.random.default_rng(505)
    n = 24
    labels, coeffs = workloads.random_pauli_sum(rng, n, 400)
    S = workloads.sample_sector(rng, 1 << 16, [(12, 6), (12, 6)])
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    terms = DeviceTerms(h)
    lf = DeviceSubspace(S, num_qubits=n, key_bits=key_bits, line_bits=line_bits)
    assert 0 < lf.c.lshift <= key_bits
    words = lf.lmap.cpu().numpy().view(np.uint32)
    ones = int(np.bitwise_count(words).sum())
    assert len(S) < ones <= 2 * len(S)                # two bits per state, a few shared
    plain = DeviceSubspace(S, num_qubits=n, key_bits=key_bits, line_filter=False)
    dt = getattr(torch, dtype)
    if not dt.is_complex and not terms.is_real:
        pytest.skip('complex coefficients need complex vectors')
    x = torch.as_tensor(rng.normal(size=len(S)) + 1j * rng.normal(size=len(S)))
    x = (x if dt.is_complex else x.real).to(dt).cuda()
    a = DeviceOperator(terms, lf, mode='free')
    y = a.matvec(x)
    a.check_errors()
    assert torch.equal(y, DeviceOperator(terms, plain, mode='free').matvec(x))
    assert torch.equal(y, DeviceOperator(terms, lf, mode='conn').matvec(x))


@pytest.mark.parametrize('line', [True, False])
def test_hash_kernel_streams_more_than_16384_groups(line):
    """A Pauli sum with more X groups than shared memory holds (the group keys are streamed in
    tiles): the matrix-free product equals the oracle's row-by-row product and, bit for bit, the
    cached-connectivity product."""
    import torch
    from oracle import sqd as osqd
    from oracle.paulis import from_paulisum as oterms
    from rqutils_gb300 import workloads
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    rng = np.random.default_rng(606)
    n = 22
    labels, coeffs = workloads.random_pauli_masks(rng, n, 60000, locality=(3, 8))
    S = workloads.sample_sector(rng, 3000, [(11, 5), (11, 6)])
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    assert len(h.xmask) > 20000
    ot = oterms((labels, coeffs), force_real=True)
    v = workloads.random_vector(rng, len(S))
    ref, hits = osqd.rows_matvec(v, ot, S, np.arange(len(S)))
    assert sum(len(r) for r in hits) > 1000
    terms = DeviceTerms(h)
    sub = DeviceSubspace(S, num_qubits=n, line_filter=line)
    free = DeviceOperator(terms, sub, mode='free')
    y = free.matvec(torch.as_tensor(v).cuda())
    free.check_errors()
    yh = y.cpu().numpy()
    assert np.linalg.norm(yh - ref) <= 1e-12 * np.linalg.norm(ref)
    assert torch.equal(y, DeviceOperator(terms, sub, mode='conn').matvec(torch.as_tensor(v).cuda()))


@pytest.mark.parametrize('variant', ['reference', 'fast'])
def test_start_almost_inside_a_two_dimensional_invariant_subspace(variant):
    """A diagonal Hamiltonian (Z terms only) from x0 = e_a + 2 e_b + 1e-9 e_c: at first the new
    search direction lies inside span(x, y) up to a relative 1e-9, where a norm taken from inner
    products is only rounding; the solver must still return the lowest of the three diagonal
    values, not a Rayleigh-Ritz value of a mis-scaled basis."""
    import torch
    from rqutils_gb300.ground_locg import lobpcg_solve
    from rqutils_gb300.sqd import SQDProblem
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    n = 6
    rng = np.random.default_rng(77)
    labels = [''.join(rng.choice(['I', 'Z'], size=n)) for _ in range(12)]
    h = PauliSumXZ.from_paulisum((labels, rng.normal(size=12)), force_real=True, add_padding=True)
    S = np.arange(1 << n, dtype=np.uint64)
    prob = SQDProblem(h, S, cache_level=(1, 0))
    d = prob.op.diag0.cpu().numpy()
    order = np.argsort(d)
    a, b, c = int(order[5]), int(order[9]), int(order[20])   # c above a and b
    assert d[a] < d[b] < d[c]
    x0 = np.zeros(1 << n)
    x0[a], x0[b], x0[c] = 1., 2., 1e-9
    eig, x, info = lobpcg_solve(prob.op, torch.as_tensor(x0).cuda(), maxiter=200,
                                variant=variant, target_rel=1e-10)
    assert np.isfinite(eig)
    assert abs(eig - d[a]) <= 1e-10 * max(1., abs(d[a])), (eig, d[a], d[b], d[c])
    assert abs(abs(x.cpu().numpy()[a]) - 1.) < 1e-8


def test_32bit_keys_with_x_masks_above_bit_31():
    """32-bit keys (every state below 2^32) with a Pauli sum on 40 qubits: targets S[i] ^ x with
    bits at or above 32 are never states, even where their low 32 bits equal one; the products
    equal the oracle's."""
    import torch
    from oracle import sqd as osqd
    from oracle.paulis import from_paulisum as oterms
    from rqutils_gb300 import workloads
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    rng = np.random.default_rng(808)
    labels, coeffs = workloads.random_pauli_masks(rng, 40, 600, locality=(1, 4))
    # terms whose X part has bits at or above 32 and whose low half alone connects states
    hi = ['X' * 2 + 'I' * 6 + lab[8:] for lab in labels[:200]]
    labels, coeffs = list(labels) + hi, np.concatenate([coeffs, rng.normal(size=200)])
    S = workloads.sample_sector(rng, 4000, [(16, 8), (16, 8)])
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    ot = oterms((labels, coeffs), force_real=True)
    assert any(int(x) >> 32 for x in h.xmask)
    terms = DeviceTerms(h)
    sub = DeviceSubspace(S, num_qubits=32, key_bits=32)
    v = workloads.random_vector(rng, len(S))
    ref, _ = osqd.rows_matvec(v, ot, S, np.arange(len(S)))
    for mode in ('free', 'conn'):
        op = DeviceOperator(terms, sub, mode=mode)
        y = op.matvec(torch.as_tensor(v).cuda()).cpu().numpy()
        assert np.linalg.norm(y - ref) <= 1e-12 * np.linalg.norm(ref), mode
