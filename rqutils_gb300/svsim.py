r"""State-vector simulation on the GPU -- drop-in for ``rqutils.svsim``.

``svsim(circuit, initial_state=0)`` and ``to_circuitxz(circuit)`` keep the reference signatures
(``rqutils/svsim.py:58-85, 131-194``): the circuit is a ``CircuitXZ``, a list of gate specifiers
``(name, qubit)`` / ``(name, qubit, angle)`` with names x, y, z, cz, rx, ry, rz, rzz, or a qiskit
``QuantumCircuit`` when qiskit is installed.  Every gate is the Pauli rotation of the reference,

    out[i] = 1j * sin * (-1)^popcount(i & z) * state[i ^ x] + cos * state[i]

applied by ``rq_svsim`` on a complex128 device state (runs of diagonal gates fused into one pass,
a non-diagonal gate one in-place pass over amplitude pairs).  The result is a torch CUDA tensor
(the reference returns a jax.Array); one GPU, so ``out_sharding`` must be None.

As in the reference, ``ry`` with a general angle maps through cos(theta/2) + sin(theta/2) Y
(the pair (x, z) = (1, 1) with the sign taken at the output index), which is not the unitary
RY(theta); ``y`` itself (theta = pi) is exact.
"""
import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from .device import default_device

try:  # optional, as in the reference
    from qiskit.circuit import QuantumCircuit
    HAS_QISKIT = True
except ImportError:
    HAS_QISKIT = False

_SPECS = {'x': (1, 0, 'pi'), 'y': (1, 1, 'pi'), 'z': (0, 1, 'pi'), 'rx': (1, 0, None),
          'ry': (1, 1, None), 'rz': (0, 1, None), 'rzz': (0, 1, None)}


@dataclass
class CircuitXZ:
    """Symplectic (XZ) representation of a series of rotation gates (svsim.py:42-49)."""
    x: np.ndarray
    z: np.ndarray
    cos: np.ndarray
    sin: np.ndarray
    num_qubits: int


def to_circuitxz(circuit):
    """Gate specifiers or a QuantumCircuit -> CircuitXZ (svsim.py:131-194): X / Z masks, and
    cos / sin of -angle / 2 (pi gates: sin = -1, cos = 0); a QuantumCircuit's cz becomes
    rzz(pi/2) rz(-pi/2) rz(-pi/2)."""
    if isinstance(circuit, CircuitXZ):
        return circuit
    num_qubits = None
    if HAS_QISKIT and isinstance(circuit, QuantumCircuit):
        def qidx(qubits):
            if isinstance(qubits, tuple):
                return np.array(list(map(circuit.qregs[0].index, qubits)))
            return np.array([circuit.qregs[0].index(qubits)])
        specs = []
        for datum in circuit.data:
            op = datum.operation
            if op.name == 'cz':
                specs.extend([('rzz', qidx(datum.qubits), np.pi / 2.),
                              ('rz', qidx(datum.qubits[0]), -np.pi / 2.),
                              ('rz', qidx(datum.qubits[1]), -np.pi / 2.)])
            elif op.params:
                specs.append((op.name, qidx(datum.qubits), op.params[0]))
            else:
                specs.append((op.name, qidx(datum.qubits)))
        num_qubits = circuit.num_qubits
        circuit = specs
    expanded = list(circuit)  # in a gate list, cz is not accepted (svsim.py:165-179)
    ng = len(expanded)
    x = np.zeros(ng, dtype=np.int64)
    z = np.zeros(ng, dtype=np.int64)
    c = np.zeros(ng, dtype=np.float64)
    s = np.zeros(ng, dtype=np.float64)
    qmax = 0
    for g, gate in enumerate(expanded):
        if gate[0] not in _SPECS:
            raise ValueError(f'Unsupported gate name {gate[0]}')
        sx, sz, ang = _SPECS[gate[0]]
        qubits = np.asarray(gate[1])
        x[g] = np.sum(np.array(sx, dtype=np.int64) << qubits)
        z[g] = np.sum(np.array(sz, dtype=np.int64) << qubits)
        if ang == 'pi':
            s[g] = -1.
        else:
            c[g] = np.cos(-gate[2] * 0.5)
            s[g] = np.sin(-gate[2] * 0.5)
        qmax = max(qmax, int(np.max(qubits)) + 1)
    return CircuitXZ(x, z, c, s, qmax if num_qubits is None else num_qubits)


def svsim(circuit, initial_state=0, out_sharding=None, *, device=None, stream=None):
    """Final state vector (complex128 torch CUDA tensor of 2^n amplitudes)."""
    if out_sharding is not None:
        raise ValueError('out_sharding: one GPU, the state is not sharded')
    circ = to_circuitxz(circuit)
    n = int(circ.num_qubits)
    dev = device or default_device()
    N = 1 << n
    if isinstance(initial_state, torch.Tensor) and initial_state.ndim == 1:
        state = initial_state.to(dev, torch.complex128).clone()
    elif np.ndim(initial_state) == 0:
        state = torch.zeros(N, dtype=torch.complex128, device=dev)
        k = int(initial_state)
        if 0 <= k < N:
            state[k] = 1.
    else:
        state = torch.as_tensor(np.asarray(initial_state, dtype=np.complex128)).to(dev)
    if state.numel() != N:
        raise ValueError(f'initial state has {state.numel()} amplitudes for {n} qubits')
    return apply_circuit(circ, state, stream=stream)


def apply_circuit(circuit, state, stream=None):
    """Apply the circuit to a complex128 device state of 2^num_qubits amplitudes in place."""
    circ = to_circuitxz(circuit)
    n = int(circ.num_qubits)
    if state.dtype != torch.complex128 or not state.is_cuda or state.numel() != (1 << n):
        raise ValueError('state must be a complex128 CUDA tensor of 2^num_qubits amplitudes')
    state = state.contiguous() if not state.is_contiguous() else state
    dev = state.device
    ng = len(circ.x)
    x = np.ascontiguousarray(circ.x, dtype=np.int64)
    z = np.ascontiguousarray(circ.z, dtype=np.int64)
    c = np.ascontiguousarray(circ.cos, dtype=np.float64)
    s = np.ascontiguousarray(circ.sin, dtype=np.float64)
    scratch = torch.empty(max(32 * ng, 32), dtype=torch.uint8, device=dev)
    L.check(L.lib().rq_svsim(x.ctypes.data, z.ctypes.data, c.ctypes.data, s.ctypes.data, ng, n,
                             L.ptr(state), L.ptr(scratch), L.stream_ptr(stream)), 'rq_svsim')
    return state
