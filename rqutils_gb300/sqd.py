r"""Sample-based quantum diagonalisation on the GPU -- drop-in for ``rqutils.sqd``.

``sqd(hamiltonian, states, states_size=None, return_eigvec=True, cache_level=(1, 0))`` and
``hproj(hamiltonian, states, unique_states=False)`` keep the reference signatures and results
(``rqutils/sqd.py:181-296``).  The Hamiltonian may be a ``PauliSumXZ``, a ``([str], [coeff])``
tuple or a qiskit ``SparsePauliOp``; ``states`` is either the reference's (D_in, n) 0/1 array
(duplicates allowed, column 0 = qubit n-1) or a sorted, distinct 1-d uint64 array (bit q = qubit q).

Pipeline (all device work in librqsqd.so):

1. terms grouped by X signature and phased (``PauliSumXZ.from_paulisum(force_real=True)``);
2. the sorted subspace: sample rows packed and deduplicated by a device radix sort
   (``uniquify_states``, sqd.py:414-445), then its hash table and sector filter (replacing the
   per-signature sorts of ``get_xsource``, sqd.py:448-503);
3. the operator in the mode ``cache_level`` asks for: (0, *) lookups in every matvec, (1, 0|1)
   cached source lists with diagonals recomputed (the reference default), (*, 2) cached elements;
4. the initial vector of sqd.py:373-398 (one-hot at the first minimum of the x = 0 diagonal);
5. LOBPCG on the device (``ground_locg``), convergence test with the vector length ``states_size``.

Keyword-only extras: ``precision`` ('fp64' default; 'mixed' runs complex64/float32 matvecs first
and refines in FP64), ``variant`` ('reference' | 'fast'), ``lookup`` ('hash' | 'bsearch'),
``maxiter``, ``tol``, ``target_rel``, ``jacobi``, ``restart`` (FAST: restart the step from x
every that many iterations of a phase; 0, the default, never, as the reference), ``return_info``.
"""
import logging
import time

import numpy as np
import torch

from .device import DeviceOperator, DeviceSubspace, DeviceTerms, default_device
from .ground_locg import lobpcg_solve
from .paulis.symplectic import PauliSumXZ

LOG = logging.getLogger(__name__)

_MODE = {0: 'free', 1: 'conn'}


def pack_states(states01):
    """(D, n) 0/1 rows -> uint64 with column 0 as qubit n-1 (sqd.py:237 without the padding bit)."""
    a = np.asarray(states01)
    n = a.shape[1]
    if n > 64:
        raise ValueError('at most 64 qubits are supported')
    w = np.left_shift(np.uint64(1), np.arange(n - 1, -1, -1, dtype=np.uint64))
    return np.bitwise_or.reduce(np.where(a.astype(bool), w, np.uint64(0)), axis=1).astype(np.uint64)


def unpack_states(states, n):
    """uint64 -> (D, n) uint8 rows (sqd.py:246)."""
    s = np.asarray(states, dtype=np.uint64)
    shifts = np.arange(n - 1, -1, -1, dtype=np.uint64)
    return ((s[:, None] >> shifts[None, :]) & np.uint64(1)).astype(np.uint8)


def subspace_states(states, num_qubits):
    """Sorted distinct uint64 states from either input form."""
    a = np.asarray(states)
    if a.ndim == 2:
        if a.shape[1] != num_qubits:
            raise ValueError(f'states have {a.shape[1]} columns for {num_qubits} qubits')
        from .workloads import sorted_unique
        return sorted_unique(pack_states(a))
    if a.ndim == 1:
        u = a.astype(np.uint64)
        if len(u) > 1 and not np.all(u[1:] > u[:-1]):
            raise ValueError('1-d uint64 states must be strictly increasing (sorted, distinct)')
        return u
    raise ValueError('states must be a (D, n) 0/1 array or a 1-d uint64 array')


def pack_states_device(states01, device=None):
    """(D, n) 0/1 rows -> int64 tensor of uint64 states on the device (rq_pack_states)."""
    import ctypes  # noqa: F401  (argument types come from _lib)
    from . import _lib as L
    a = np.ascontiguousarray(np.asarray(states01), dtype=np.uint8)
    rows, n = a.shape
    if n > 64:
        raise ValueError('at most 64 qubits are supported')
    dev = device or default_device()
    bits = torch.from_numpy(a).to(dev)
    out = torch.empty(rows, dtype=torch.int64, device=dev)
    L.check(L.lib().rq_pack_states(L.ptr(bits), rows, n, n, L.ptr(out), L.stream_ptr()),
            'rq_pack_states')
    return out


def uniquify_device(packed):
    """Sorted distinct values of a device tensor of uint64 samples (rq_uniquify)."""
    import ctypes
    from . import _lib as L
    packed = packed.contiguous()
    n = packed.numel()
    nb = ctypes.c_size_t()
    L.check(L.lib().rq_uniquify_scratch_size(n, ctypes.byref(nb)), 'rq_uniquify_scratch_size')
    scratch = torch.empty(int(nb.value), dtype=torch.uint8, device=packed.device)
    out = torch.empty_like(packed)
    cnt = ctypes.c_int64()
    L.check(L.lib().rq_uniquify(L.ptr(packed), n, L.ptr(out), ctypes.byref(cnt), L.ptr(scratch),
                                L.stream_ptr()), 'rq_uniquify')
    return out[:cnt.value]


def subspace_states_device(states, num_qubits, device=None):
    """Sorted distinct states on the device from either input form: (D_in, n) 0/1 rows are
    packed and deduplicated by the device radix sort; a 1-d uint64 array is checked for strict
    increase.  Returns (int64 device tensor, uint64 host array)."""
    a = np.asarray(states)
    dev = device or default_device()
    if a.ndim == 2:
        if a.shape[1] != num_qubits:
            raise ValueError(f'states have {a.shape[1]} columns for {num_qubits} qubits')
        S = uniquify_device(pack_states_device(a, dev))
        return S, S.cpu().numpy().view(np.uint64)
    u = subspace_states(a, num_qubits)
    return torch.from_numpy(u.view(np.int64)).to(dev), u


def cache_mode(cache_level):
    c0, c1 = cache_level
    if c1 == 2:
        return 'csr'
    if c0 not in (0, 1) or c1 not in (0, 1):
        raise ValueError(f'unsupported cache_level {cache_level}')
    return _MODE[c0]


class SQDProblem:
    """Hamiltonian terms and subspace on the device with the operator built for cache_level."""

    def __init__(self, hamiltonian, states_u64, cache_level=(1, 0), lookup='hash',
                 filter_masks=None, device=None, precision='fp64', line_bits=8, tune_cache=None):
        """``cache_level='auto'``: the form of the product (matrix-free with or without the line
        filter, binary search, cached connectivity or elements) is chosen by measurement
        (``rqutils_gb300.autotune.tune``, recorded per problem class in ``tune_cache``)."""
        self.device = device or default_device()
        self.ham = hamiltonian
        self.n = hamiltonian.num_qubits
        self.states = states_u64
        line_filter = True
        if cache_level == 'auto':
            from .autotune import tune
            single = precision == 'fp32'
            if hamiltonian.is_real:
                dt = torch.float32 if single else torch.float64
            else:
                dt = torch.complex64 if single else torch.complex128
            (mode, lookup, lb), _ = tune(hamiltonian, states_u64, dtype=dt, cache=tune_cache,
                                         device=self.device)
            line_filter, line_bits = lb > 0, lb or 8
            cache_level = {'free': (0, 0), 'conn': (1, 0), 'csr': (1, 2)}[mode]
        self.cache_level = cache_level
        self.terms = DeviceTerms(hamiltonian, device=self.device)
        self.sub = DeviceSubspace(states_u64, num_qubits=self.n, lookup=lookup,
                                  filter_masks=filter_masks, device=self.device,
                                  line_filter=line_filter, line_bits=line_bits)
        mode = cache_mode(cache_level)
        csr_vtype = None
        if mode == 'csr':
            from .device import vtype_for
            csr_vtype = vtype_for(self.terms.is_real, 'fp32' if precision == 'fp32' else 'fp64')
        self.op = DeviceOperator(self.terms, self.sub, mode=mode, csr_vtype=csr_vtype)
        self.dtype = torch.float64 if self.terms.is_real else torch.complex128

    def initial_vector(self, dtype=None):
        """sqd.py:373-398: one-hot at the first minimum of the x = 0 group's diagonal when group 0
        is that group, else at index 0."""
        dtype = dtype or self.dtype
        x0 = torch.zeros(self.sub.D, dtype=dtype, device=self.device)
        if self.terms.diag_group == 0 and self.op.diag0 is not None:
            x0[int(torch.argmin(self.op.diag0))] = 1
        else:
            x0[0] = 1
        return x0


def sqd(hamiltonian, states, states_size=None, return_eigvec=True, cache_level=(1, 0), *,
        precision='fp64', variant='reference', lookup='hash', maxiter=1000, tol=None,
        target_rel=None, jacobi=False, use_graph=True, restart=0, return_info=False,
        device=None):
    """Ground eigenpair of the Hamiltonian projected on the subspace spanned by ``states``.

    ``cache_level`` is the reference's (0, *), (1, 0|1) or (*, 2), or ``'auto'`` (not in the
    reference): the form of the product chosen by measurement (``rqutils_gb300.autotune``).

    Returns the energy, or ``(energy, eigvec (D,), basis_states (D, n) uint8)`` with
    ``return_eigvec`` (sqd.py:243-248); ``return_info`` appends a dict of solver statistics.
    """
    n_in = np.asarray(states).shape[0]
    if states_size is None:
        states_size = n_in
    if states_size < n_in:
        raise ValueError('states_size smaller than the states array length')
    if not isinstance(hamiltonian, PauliSumXZ):
        hamiltonian = PauliSumXZ.from_paulisum(hamiltonian, force_real=True, add_padding=True)
    start = time.time()
    S_dev, S = subspace_states_device(states, hamiltonian.num_qubits, device)
    prob = SQDProblem(hamiltonian, S_dev, cache_level=cache_level, lookup=lookup, device=device,
                      precision=precision)
    x0 = prob.initial_vector()
    eig, x, info = lobpcg_solve(prob.op, x0, maxiter=maxiter, tol=tol, tol_dim=states_size,
                                variant=variant, mixed=(precision == 'mixed'),
                                target_rel=target_rel, jacobi=jacobi, use_graph=use_graph,
                                restart=restart)
    LOG.info('Found ground eigenpair in %f seconds.', time.time() - start)
    eigval = float(eig)
    if not return_eigvec:
        return (eigval, info) if return_info else eigval
    out = (eigval, x.cpu().numpy(), unpack_states(S, hamiltonian.num_qubits))
    return out + (info,) if return_info else out


def hproj(hamiltonian, states, unique_states=False, *, device=None):
    """The Hamiltonian projected onto the subspace as a scipy CSR matrix (sqd.py:251-296):
    rows / columns in the sorted order of the unique states, elements from every X group
    including the diagonal one.  (The Hamiltonian is not forced real, as in the reference.)"""
    from scipy.sparse import csr_array, coo_array
    if not isinstance(hamiltonian, PauliSumXZ):
        hamiltonian = PauliSumXZ.from_paulisum(hamiltonian, add_padding=True)
    a = np.asarray(states)
    if a.ndim == 2:
        from .workloads import sorted_unique
        S = pack_states(a)
        S = sorted_unique(S) if not unique_states else S
    else:
        S = a.astype(np.uint64)
    prob = SQDProblem(hamiltonian, S, cache_level=(1, 2), device=device)
    op = prob.op
    rowptr = op.rowptr.cpu().numpy()
    cols = op.col[:op.nnz].cpu().numpy()
    vals = op.val[:op.nnz].cpu().numpy()
    D = len(S)
    rows = np.repeat(np.arange(D), np.diff(rowptr))
    if op.diag0 is not None:
        dg = prob.op.group_diagonal(prob.terms.diag_group).cpu().numpy()
        rows = np.concatenate([np.arange(D), rows])
        cols = np.concatenate([np.arange(D), cols])
        vals = np.concatenate([dg.astype(vals.dtype) if np.iscomplexobj(vals) else dg.real, vals])
    return csr_array(coo_array((vals, (rows, cols)), shape=(D, D)))
