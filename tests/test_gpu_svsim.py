"""State-vector simulation (rq_svsim) against the oracle's restatement of the reference
arithmetic (bit for bit) and against dense rotation matrices."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _random_circuit(rng, n, ngates):
    names = ['x', 'y', 'z', 'rx', 'ry', 'rz', 'rzz']
    circ = []
    for _ in range(ngates):
        name = names[rng.integers(len(names))]
        if name == 'rzz':
            q = rng.choice(n, size=2, replace=False)
            circ.append((name, q, rng.uniform(-np.pi, np.pi)))
        elif name.startswith('r'):
            circ.append((name, int(rng.integers(n)), rng.uniform(-np.pi, np.pi)))
        else:
            circ.append((name, int(rng.integers(n))))
    return circ


@pytest.mark.parametrize('n,ngates', [(1, 5), (6, 40), (12, 300), (20, 60)])
def test_svsim_bit_exact_against_oracle(n, ngates):
    from oracle import svsim as osv
    from rqutils_gb300.svsim import svsim, to_circuitxz
    rng = np.random.default_rng(n * 100 + ngates)
    circ = _random_circuit(rng, n, ngates)
    cx = to_circuitxz(circ)
    ox, oz, oc, os_, on = osv.to_circuitxz(circ)
    np.testing.assert_array_equal(cx.x, ox)
    np.testing.assert_array_equal(cx.z, oz)
    np.testing.assert_array_equal(cx.cos, oc)
    np.testing.assert_array_equal(cx.sin, os_)
    assert cx.num_qubits == on
    psi0 = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    for init in (0, 3 % (2 ** n), psi0):
        got = svsim(circ, initial_state=init).cpu().numpy()
        ref = osv.svsim(ox, oz, oc, os_, on, initial_state=init)
        assert np.array_equal(got, ref), np.max(np.abs(got - ref))


def _pauli(label):
    m = {'I': np.eye(2), 'X': np.array([[0, 1], [1, 0]]), 'Y': np.array([[0, -1j], [1j, 0]]),
         'Z': np.diag([1., -1.])}
    out = np.array([[1.]])
    for ch in label:
        out = np.kron(out, m[ch])
    return out


@pytest.mark.parametrize('name,qubits,angle,label,phase', [
    ('rx', 0, 0.7, 'IIX', None), ('rz', 2, -1.1, 'ZII', None), ('rzz', [0, 2], 0.4, 'ZIZ', None),
    ('x', 1, None, 'IXI', -1j), ('y', 1, None, 'IYI', 1.), ('z', 0, None, 'IIZ', -1j)])
def test_rotations_match_dense_exponentials(name, qubits, angle, label, phase):
    """Unitary gates of the set: exp(-i theta/2 P); the pi gates are P times the reference's
    global phase (-i for x and z, 1 for y)."""
    import scipy.linalg
    from rqutils_gb300.svsim import svsim, to_circuitxz
    rng = np.random.default_rng(5)
    psi = rng.normal(size=8) + 1j * rng.normal(size=8)
    spec = (name, qubits) if angle is None else (name, qubits, angle)
    circ = to_circuitxz([spec])
    circ.num_qubits = 3
    got = svsim(circ, initial_state=psi).cpu().numpy()
    P = _pauli(label)
    U = phase * P if angle is None else scipy.linalg.expm(-0.5j * angle * P)
    np.testing.assert_allclose(got, U @ psi, rtol=1e-12, atol=1e-12)


def test_reference_errors():
    from rqutils_gb300.svsim import svsim
    with pytest.raises(ValueError):
        svsim([('cz', [0, 1])])
    with pytest.raises(ValueError):
        svsim([('h', 0)])


@pytest.mark.parametrize('name', __import__('golden_cases').svsim_case_names())
def test_svsim_matches_reference_fixtures(name):
    """rq_svsim against final states recorded from the unmodified reference rqutils/svsim.py:
    bit for bit (values compared with ==, so only the sign of a zero may differ)."""
    from golden_cases import load_svsim
    from rqutils_gb300.svsim import svsim
    d = load_svsim(name)
    init = d['initial'] if d['initial'].ndim else int(d['initial'])
    got = svsim(d['circuit'], init)
    np.testing.assert_array_equal(got.cpu().numpy(), d['final'])
