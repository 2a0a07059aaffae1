"""Batched SQD (rq_batch_*) against the reference fixtures, the oracle and single-problem runs."""
import warnings

import numpy as np
import pytest

from golden_cases import case_names, hamiltonian, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _golden_batch(cache_level):
    from rqutils_gb300.batch import BatchedSQD
    cases = [load(n) for n in case_names()]
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        b = BatchedSQD([hamiltonian(c) for c in cases], [c['states'] for c in cases],
                       cache_level=cache_level,
                       states_sizes=[int(c['states_size']) for c in cases])
    return b, cases


def _random_problems(seed, P, n_range=(8, 40), d_range=(64, 4096), k_range=(20, 300)):
    from rqutils_gb300.workloads import batched_random_problems
    return batched_random_problems(seed, P=P, n_range=n_range, k_range=k_range, d_range=d_range)


@pytest.mark.parametrize('cache_level', [(0, 0), (1, 0)])
def test_batch_matvec_matches_reference_outputs(cache_level):
    """One launch over every fixture problem reproduces each problem's reference matvec."""
    import torch
    b, cases = _golden_batch(cache_level)
    dt = torch.float64 if b.is_real else torch.complex128
    for k in range(len(cases[0]['mv_in'])):
        x = torch.cat([torch.as_tensor(c['mv_in'][k][:int(c['D'])]).to(dt) for c in cases]).cuda()
        y = b.matvec(x).cpu().numpy()
        b.check_errors()
        for p, c in enumerate(cases):
            ref = c['mv_out'][k][:int(c['D'])]
            got = y[b.rows(p)]
            if not np.iscomplexobj(ref):
                assert np.all(got.imag == 0) if np.iscomplexobj(got) else True
                got = got.real
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize('cache_level', [(0, 0), (1, 0)])
def test_batch_sqd_matches_reference(cache_level):
    """Every fixture problem solved in one batch: the reference's eigenpair, basis and iteration
    count (NaN outcomes of the reference included)."""
    from rqutils_gb300.batch import sqd_batch
    cases = [load(n) for n in case_names()]
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        out, infos = sqd_batch([hamiltonian(c) for c in cases], [c['states'] for c in cases],
                               states_sizes=[int(c['states_size']) for c in cases],
                               cache_level=cache_level, return_info=True)
    for (eig, vec, basis), info, c in zip(out, infos, cases):
        ref = float(c['eigval'])
        np.testing.assert_array_equal(basis, c['basis'])
        if np.isnan(ref):
            assert np.isnan(eig) and info['niter'] == int(c['niter'])
            continue
        assert abs(eig - ref) <= 1e-10 * max(1., abs(ref)), (eig, ref)
        assert abs(np.vdot(c['eigvec'].astype(np.complex128), vec)) > 1 - 1e-9
        assert abs(info['niter'] - int(c['niter'])) <= max(2, int(0.05 * int(c['niter'])))


def test_batch_matvec_random_vs_single_and_oracle():
    """Random problems up to 40 qubits: batched FREE and CONN products equal the single-problem
    kernels' and the oracle's."""
    import torch
    from oracle.paulis import from_paulisum as o_from
    from oracle.sqd import matvec_nocache
    from rqutils_gb300.batch import BatchedSQD
    from rqutils_gb300.sqd import SQDProblem
    hams, states, ns = _random_problems(11, 12)
    rng = np.random.default_rng(3)
    for cache_level in [(0, 0), (1, 0)]:
        b = BatchedSQD(hams, states, cache_level=cache_level)
        x = torch.as_tensor(rng.normal(size=b.D) + 1j * rng.normal(size=b.D)).cuda()
        y = b.matvec(x).cpu().numpy()
        b.check_errors()
        for p in range(b.P):
            single = SQDProblem(b.hams[p], states[p], cache_level=cache_level)
            ys = single.op.matvec(x[b.rows(p)].contiguous()).cpu().numpy()
            np.testing.assert_allclose(y[b.rows(p)], ys, rtol=1e-13, atol=1e-13)
            if p < 3:
                t = o_from(hams[p], force_real=True)
                yo = matvec_nocache(x[b.rows(p)].cpu().numpy(), t, states[p])
                np.testing.assert_allclose(y[b.rows(p)], yo, rtol=1e-11, atol=1e-11)


def test_batch_matvec_fp32_error_bound():
    import torch
    from rqutils_gb300.batch import BatchedSQD
    hams, states, ns = _random_problems(12, 8)
    b = BatchedSQD(hams, states, cache_level=(0, 0))
    rng = np.random.default_rng(4)
    x = torch.as_tensor(rng.normal(size=b.D) + 1j * rng.normal(size=b.D)).to(torch.complex64).cuda()
    y = b.matvec(x).cpu().numpy()
    exact = b.matvec(x.to(torch.complex128)).cpu().numpy()
    for p in range(b.P):
        r = b.rows(p)
        e = np.linalg.norm(y[r] - exact[r]) / max(np.linalg.norm(exact[r]), 1e-300)
        assert e <= 1e-6, (p, e)


@pytest.mark.parametrize('variant', ['reference', 'fast'])
def test_batch_solve_matches_single_solves(variant):
    """Batched LOBPCG = the single-problem solver on each problem (same start vector and
    convergence length)."""
    import torch
    from rqutils_gb300.batch import BatchedSQD
    from rqutils_gb300.ground_locg import lobpcg_solve
    from rqutils_gb300.sqd import SQDProblem, sqd
    hams, states, ns = _random_problems(13, 10)
    b = BatchedSQD(hams, states, cache_level=(0, 0))
    # the sqd() start vector (a one-hot that can sit on an isolated row: NaN, as the reference)
    eig, x, infos = b.solve(variant=variant)
    xs = x.cpu().numpy()
    nan = 0
    for p in range(b.P):
        e1, v1, _, info1 = sqd(b.hams[p], states[p], variant=variant, cache_level=(0, 0),
                               return_info=True)
        assert infos[p]['niter'] == info1['niter'] or abs(infos[p]['niter'] - info1['niter']) <= 2
        if np.isnan(e1):
            assert np.isnan(eig[p])
            nan += 1
            continue
        assert abs(eig[p] - e1) <= 1e-10 * max(1., abs(e1)), (p, eig[p], e1)
        assert infos[p]['converged'] == info1['converged']
        assert abs(np.vdot(v1, xs[b.rows(p)])) > 1 - 1e-8
    assert nan < b.P  # sparse random subspaces: many one-hot starts are isolated rows
    # a random start: every problem converges, as it does alone
    rng = np.random.default_rng(21)
    xr = rng.normal(size=b.D) + 1j * rng.normal(size=b.D)
    x0 = torch.as_tensor(xr.real if b.is_real else xr).to(b.dtype).cuda()
    eig, x, infos = b.solve(x0=x0, variant=variant)
    xs = x.cpu().numpy()
    for p in range(b.P):
        single = SQDProblem(b.hams[p], states[p], cache_level=(0, 0))
        e1, v1, info1 = lobpcg_solve(single.op, x0[b.rows(p)].contiguous(), variant=variant)
        v1 = v1.cpu().numpy()
        assert infos[p]['converged'] and info1['converged']
        assert abs(eig[p] - e1) <= 1e-10 * max(1., abs(e1)), (p, eig[p], e1)
        assert abs(infos[p]['niter'] - info1['niter']) <= 2, (p, infos[p], info1)
        assert abs(np.vdot(v1, xs[b.rows(p)])) > 1 - 1e-8


def test_batch_solve_oracle_eigenvalues():
    """Ground energies of small batched problems against the oracle's LOBPCG and the dense
    projected matrix."""
    from oracle.dense import projected_ground
    from oracle.sqd import sqd as o_sqd
    from rqutils_gb300.batch import sqd_batch
    hams, states, ns = _random_problems(14, 6, n_range=(8, 10), d_range=(32, 400),
                                        k_range=(20, 80))
    import torch
    from rqutils_gb300.batch import BatchedSQD
    out = sqd_batch(hams, states, return_eigvec=False)
    for p in range(len(hams)):
        eo = o_sqd(hams[p], states[p], return_eigvec=False)
        if np.isnan(eo):  # the reference's one-hot start on an isolated row
            assert np.isnan(out[p])
            continue
        assert abs(out[p] - eo) <= 1e-9 * max(1., abs(eo)), (p, out[p], eo)
    # a one-hot start stays in its connected block of a sparse subspace; from a random start
    # every problem reaches the ground energy of its whole projected matrix
    b = BatchedSQD(hams, states)
    xr = np.random.default_rng(8).normal(size=b.D) + 1j * np.random.default_rng(9).normal(size=b.D)
    eig, _, _ = b.solve(x0=torch.as_tensor(xr.real if b.is_real else xr).to(b.dtype).cuda())
    for p in range(len(hams)):
        ed = projected_ground(hams[p][0], hams[p][1], states[p])[0]
        assert abs(eig[p] - ed) <= 1e-8 * max(1., abs(ed)), (p, eig[p], ed)


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_batch_solve_low_precision(precision):
    from rqutils_gb300.batch import BatchedSQD
    import torch
    hams, states, ns = _random_problems(15, 8)
    b = BatchedSQD(hams, states, cache_level=(0, 0))
    rng = np.random.default_rng(5)
    xr = rng.normal(size=b.D) + 1j * rng.normal(size=b.D)
    x0 = torch.as_tensor(xr.real if b.is_real else xr).to(b.dtype).cuda()
    e64, _, _ = b.solve(x0=x0)
    if precision == 'fp32':
        x0 = x0.to(torch.complex64 if x0.is_complex() else torch.float32)
    e, x, infos = b.solve(x0=x0, precision=precision)
    if precision == 'fp32':
        # the reference criterion with the 32-bit epsilon stops early on these sizes: the
        # Rayleigh quotient is still an upper bound of the FP64 ground energy
        assert np.all(e >= e64 - 1e-5 * np.abs(e64)) and np.all(e - e64 <= 5e-2 * np.abs(e64))
        assert all(i['converged'] for i in infos)
    else:
        np.testing.assert_allclose(e, e64, rtol=1e-10, atol=1e-10)
    if precision == 'mixed':
        assert any(i['niter_lo'] > 0 for i in infos)


def test_batch_rejects_wide_problems_and_bad_rows():
    import torch
    from rqutils_gb300 import _lib as L
    from rqutils_gb300.batch import BatchedSQD
    hams, states, ns = _random_problems(16, 3)
    wide = (['X' + 'I' * 40], np.array([1.0]))
    with pytest.raises(ValueError):
        BatchedSQD([wide], [np.array([0, 1], np.uint64)])
    b = BatchedSQD(hams, states, cache_level=(0, 0))
    # row ranges that disagree with the keys' problem ids are rejected by the library
    bad = torch.tensor([0, 1, b.D - 1, b.D], dtype=torch.int64, device='cuda')
    c = L.Batch.from_buffer_copy(b.c)
    c.prow = L.ptr(bad)
    import ctypes
    rc = L.lib().rq_batch_build(ctypes.byref(c), L.ptr(b.scratch), L.stream_ptr())
    assert rc == L.E_ARG


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('variant', ['reference', 'fast'])
def test_batch_persistent_launches_match_graph_chunks(variant, precision):
    """Cached-connectivity batches run each phase as persistent launches (every problem on its own
    group of blocks, re-planned every 256 iterations); the CUDA-graph chunks run the same
    iteration: same eigenvalues and eigenvectors, iteration counts within one in FP64.  With a
    32-bit phase the two block layouts add the FP32 partial sums in different orders, which can
    move the switch to FP64 by some iterations (10 % here) and the final vectors within the
    residual test."""
    import torch
    from rqutils_gb300.batch import BatchedSQD
    hams, states, ns = _random_problems(31, 40, d_range=(64, 20000))
    b = BatchedSQD(hams, states, cache_level=(1, 0))
    rng = np.random.default_rng(32)
    xr = rng.normal(size=b.D) + 1j * rng.normal(size=b.D)
    x0 = torch.as_tensor(xr.real if b.is_real else xr).to(b.dtype).cuda()
    e1, x1, i1 = b.solve(x0=x0, variant=variant, precision=precision, maxiter=3000, use_graph=1)
    e2, x2, i2 = b.solve(x0=x0, variant=variant, precision=precision, maxiter=3000, use_graph=2)
    x1, x2 = x1.cpu().numpy(), x2.cpu().numpy()
    assert max(i['niter'] for i in i1) > 256          # some problem spans several launches
    for p in range(b.P):
        assert i1[p]['converged'] == i2[p]['converged'], p
        slack = 1 if precision == 'fp64' else max(2, int(0.1 * i2[p]['niter']))
        assert abs(i1[p]['niter'] - i2[p]['niter']) <= slack, (p, i1[p], i2[p])
        if np.isnan(e2[p]):  # the same breakdown on both paths
            assert np.isnan(e1[p]), p
            continue
        assert abs(e1[p] - e2[p]) <= 1e-12 * max(1., abs(e2[p])), (p, e1[p], e2[p])
        r = b.rows(p)
        # both vectors meet the residual test, so they agree to about (residual / gap)^2
        assert abs(np.vdot(x1[r], x2[r])) > 1 - (1e-10 if precision == 'fp64' else 1e-8), p
