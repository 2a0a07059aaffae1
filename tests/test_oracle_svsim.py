"""The state-vector oracle (restatement of svsim.py) against dense rotation matrices, and the
package's circuit conversion against the oracle's (CPU)."""
import numpy as np
import pytest
import scipy.linalg

from oracle import svsim as osv

_M = {'I': np.eye(2), 'X': np.array([[0, 1], [1, 0]]), 'Y': np.array([[0, -1j], [1j, 0]]),
      'Z': np.diag([1., -1.])}


def _pauli(label):
    out = np.array([[1.]])
    for ch in label:
        out = np.kron(out, _M[ch])
    return out


@pytest.mark.parametrize('spec,label,phase', [
    (('rx', 0, 0.7), 'IIX', None), (('rz', 2, -1.1), 'ZII', None),
    (('rzz', [0, 2], 0.4), 'ZIZ', None), (('x', 1), 'IXI', -1j), (('y', 1), 'IYI', 1.),
    (('z', 0), 'IIZ', -1j)])
def test_oracle_gates_are_rotations(spec, label, phase):
    rng = np.random.default_rng(5)
    psi = rng.normal(size=8) + 1j * rng.normal(size=8)
    x, z, c, s, n = osv.to_circuitxz([spec], 3)
    P = _pauli(label)
    U = phase * P if phase is not None else scipy.linalg.expm(-0.5j * spec[2] * P)
    np.testing.assert_allclose(osv.svsim(x, z, c, s, 3, psi), U @ psi, atol=1e-12)


def test_oracle_ry_is_the_reference_map():
    """ry(theta) of the reference: cos(theta/2) I + sin(theta/2) Y (not the unitary RY)."""
    rng = np.random.default_rng(6)
    psi = rng.normal(size=2) + 1j * rng.normal(size=2)
    th = 0.9
    x, z, c, s, n = osv.to_circuitxz([('ry', 0, th)])
    ref = (np.cos(th / 2) * np.eye(2) + np.sin(th / 2) * _M['Y']) @ psi
    np.testing.assert_allclose(osv.svsim(x, z, c, s, 1, psi), ref, atol=1e-12)


def test_circuit_conversion_matches_oracle():
    from rqutils_gb300.svsim import CircuitXZ, to_circuitxz
    circ = [('x', 0), ('ry', 3, 0.3), ('rzz', [1, 4], -0.2), ('z', 2), ('rx', 1, 2.0), ('y', 4)]
    a = to_circuitxz(circ)
    x, z, c, s, n = osv.to_circuitxz(circ)
    np.testing.assert_array_equal(a.x, x)
    np.testing.assert_array_equal(a.z, z)
    np.testing.assert_array_equal(a.cos, c)
    np.testing.assert_array_equal(a.sin, s)
    assert a.num_qubits == n == 5
    assert to_circuitxz(a) is a and isinstance(a, CircuitXZ)
    with pytest.raises(ValueError):
        to_circuitxz([('cz', [0, 1])])


@pytest.mark.parametrize('name', __import__('golden_cases').svsim_case_names())
def test_oracle_matches_reference_svsim_fixtures(name):
    """The oracle restatement against outputs of the unmodified reference rqutils/svsim.py
    (recorded through the NumPy stand-in for jax): circuit arrays and final states bit for bit."""
    from golden_cases import load_svsim
    from rqutils_gb300.svsim import to_circuitxz
    d = load_svsim(name)
    x, z, c, s, n = osv.to_circuitxz(d['circuit'])
    for got, want in ((x, d['x']), (z, d['z']), (c, d['cos']), (s, d['sin'])):
        np.testing.assert_array_equal(got, want)
    assert n == int(d['num_qubits'])
    cx = to_circuitxz(d['circuit'])
    for got, want in ((cx.x, d['x']), (cx.z, d['z']), (cx.cos, d['cos']), (cx.sin, d['sin'])):
        np.testing.assert_array_equal(got, want)
    init = d['initial'] if d['initial'].ndim else int(d['initial'])
    np.testing.assert_array_equal(osv.svsim(x, z, c, s, n, init), d['final'])
