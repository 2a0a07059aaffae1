"""PauliSumXZ.from_paulisum with the consolidation, grouping and phasing on the device
(rq_terms_group) against the host path and the reference fixtures (GPU)."""
import warnings

import numpy as np
import pytest

from golden_cases import case_names, hamiltonian, load, packed_to_u64

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _same(a, b):
    np.testing.assert_array_equal(a.xmask, b.xmask)
    np.testing.assert_array_equal(a.toff, b.toff)
    np.testing.assert_array_equal(a.zmask, b.zmask)
    assert a.coef.dtype == b.coef.dtype
    np.testing.assert_array_equal(a.coef, b.coef)
    assert a.num_qubits == b.num_qubits and a.padded == b.padded


@pytest.mark.parametrize('name', case_names())
def test_device_grouping_matches_reference_fixtures(name):
    """Packed X / Z arrays equal the reference's own (recorded) arrays, the phased coefficients
    to 1e-15 (the reference merges duplicates by a matrix product, masks @ coeffs at
    symplectic.py:72, whose summation order is the BLAS library's; both paths here add them in
    input order and agree with each other bit for bit)."""
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        h = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True, add_padding=True,
                                     device='cuda')
        host = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True, add_padding=True)
    _same(h, host)
    np.testing.assert_array_equal(h.x, case['ham_x'])
    np.testing.assert_array_equal(h.z, case['ham_z'])
    assert h.c.dtype == case['ham_c'].dtype
    np.testing.assert_allclose(h.c, case['ham_c'], atol=1e-15, rtol=0)


@pytest.mark.parametrize('force_real', [False, True])
@pytest.mark.parametrize('n,K,dup', [(6, 200, 0.5), (20, 3000, 0.2), (33, 5000, 0.3),
                                     (64, 20000, 0.1)])
def test_device_grouping_matches_host(n, K, dup, force_real):
    """Random labels with duplicates (some cancelling exactly), zeros and complex coefficients."""
    from rqutils_gb300 import workloads
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    rng = np.random.default_rng(n * 7 + K)
    labels, coeffs = workloads.random_pauli_masks(rng, n, K, locality=(1, min(n, 6)))
    labels = list(labels)
    coeffs = coeffs + 1j * rng.normal(size=K) * (rng.random(K) < 0.3)
    ndup = int(dup * K)
    pick = rng.choice(K, size=ndup)
    labels += [labels[i] for i in pick]
    extra = rng.normal(size=ndup)
    extra[: ndup // 4] = -coeffs[pick[: ndup // 4]]          # exact cancellations
    coeffs = np.concatenate([coeffs, extra])
    coeffs[rng.choice(len(coeffs), size=len(coeffs) // 20)] = 0.
    with warnings.catch_warnings(record=True) as w_dev:
        warnings.simplefilter('always')
        d = PauliSumXZ.from_paulisum((labels, coeffs), force_real=force_real, device='cuda')
    with warnings.catch_warnings(record=True) as w_host:
        warnings.simplefilter('always')
        h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=force_real)
    _same(d, h)
    assert len(w_dev) == len(w_host)


def test_device_grouping_chemistry_terms():
    """The 64-qubit, 50,000-term chemistry Hamiltonian of the benchmark, real coefficients."""
    from rqutils_gb300 import workloads
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    p, c = workloads.chemistry_jw(12, np.random.default_rng(4), keep=20000)
    _same(PauliSumXZ.from_paulisum((p, c), force_real=True, add_padding=True, device='cuda'),
          PauliSumXZ.from_paulisum((p, c), force_real=True, add_padding=True))


def test_device_grouping_all_zero_and_errors():
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    d = PauliSumXZ.from_paulisum((['XI', 'ZZ'], [0., 0.]), device='cuda')
    h = PauliSumXZ.from_paulisum((['XI', 'ZZ'], [0., 0.]))
    assert len(d.xmask) == len(h.xmask) == 0 and d.coef.dtype == h.coef.dtype
    with pytest.raises(ValueError):
        PauliSumXZ.from_paulisum((['XI', 'Z'], [1., 1.]), device='cuda')
    with pytest.raises(ValueError):
        PauliSumXZ.from_paulisum((['XI'], [1., 1.]), device='cuda')
