"""Oracle (test infrastructure only): NumPy restatement of the reference state-vector simulator.

``rqutils/svsim.py:131-194`` (``to_circuitxz``: gate specs to X / Z masks and cos / sin of
-angle / 2, pi gates as sin = -1, cos = 0) and ``svsim.py:88-122`` (``do_svsim``: one-hot or given
initial state; per gate out = 1j * sin * signs * state[i ^ x] + cos * state, the cos term skipped
when cos == 0, signs = (-1)^popcount(i & z)).  The complex products are written out in NumPy's
own evaluation order so that the device kernel, which rounds each product and sum separately,
can be compared bit for bit.

Parity pin: ``tests/golden/svsim_*.npz`` hold circuits run through the unmodified reference
``rqutils/svsim.py`` (``tests/golden/make_golden.py --svsim``, jax replaced by the NumPy stand-in);
``tests/test_oracle_svsim.py`` checks this restatement against them bit for bit.
"""
import numpy as np

_SPECS = {'x': (1, 0, 'pi'), 'y': (1, 1, 'pi'), 'z': (0, 1, 'pi'), 'rx': (1, 0, None),
          'ry': (1, 1, None), 'rz': (0, 1, None), 'rzz': (0, 1, None)}


def to_circuitxz(circuit, num_qubits=None):
    """List of (name, qubit(s)[, angle]) -> (x, z, cos, sin, num_qubits) (svsim.py:154-194)."""
    ng = len(circuit)
    x = np.zeros(ng, dtype=np.int64)
    z = np.zeros(ng, dtype=np.int64)
    c = np.zeros(ng, dtype=np.float64)
    s = np.zeros(ng, dtype=np.float64)
    qmax = 0
    for g, gate in enumerate(circuit):
        if gate[0] not in _SPECS:
            raise ValueError(f'Unsupported gate name {gate[0]}')
        sx, sz, ang = _SPECS[gate[0]]
        q = np.asarray(gate[1])
        x[g] = np.sum(np.array(sx, dtype=np.int64) << q)
        z[g] = np.sum(np.array(sz, dtype=np.int64) << q)
        if ang == 'pi':
            s[g] = -1.
        else:
            c[g] = np.cos(-gate[2] * 0.5)
            s[g] = np.sin(-gate[2] * 0.5)
        qmax = max(qmax, int(np.max(q)) + 1)
    return x, z, c, s, (qmax if num_qubits is None else num_qubits)


def svsim(x, z, c, s, num_qubits, initial_state=0):
    idx = np.arange(2 ** num_qubits, dtype=np.int64)
    if np.ndim(initial_state) == 0:
        state = (idx == initial_state).astype(np.complex128)
    else:
        state = np.asarray(initial_state, dtype=np.complex128).copy()
    for xg, zg, cg, sg in zip(x, z, c, s):
        signs = 1. - 2. * (np.bitwise_count(idx & zg) & 1)
        xs = state if xg == 0 else state[idx ^ xg]
        a = sg * signs
        re = 0. * xs.real - a * xs.imag
        im = 0. * xs.imag + a * xs.real
        if cg != 0.:
            re = re + cg * state.real
            im = im + cg * state.imag
        state = re + 1j * im
    return state
