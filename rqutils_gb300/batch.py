r"""Many independent SQD problems solved together on one GPU (``rq_batch_*``).

The reference solves one problem per ``sqd()`` call (``rqutils/sqd.py:181-248``, LOBPCG in
``rqutils/ground_locg.py:182-377``).  ``BatchedSQD`` holds P problems -- each its own Pauli sum on
its own sorted subspace of at most 40 qubits -- in one set of device arrays:

* rows of every problem in one vector, problem p at rows ``prow[p] .. prow[p+1]``;
* composite keys ``(p << 40) | state`` in one sorted array and one hash table (the lookup hash is
  GF(2)-linear, so a probe of ``key ^ x`` costs what it costs for one problem);
* every problem's X groups concatenated, problem p owning groups ``gofs[p] .. gofs[p+1]``.

One matvec launch serves all problems; LOBPCG keeps per-problem reductions, Rayleigh-Ritz and
convergence, and a problem that converged drops out of the matvec and vector passes.  Each
problem's result equals ``sqd()`` on that problem alone (same start, same iteration, its own
``states_size`` in the convergence test).
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from .device import (TORCH_DTYPE, VTYPE_OF, _u64_tensor, default_device, default_filter_masks,
                     scratch_tensor, vtype_for)
from .ground_locg import _info, _params
from .paulis.symplectic import PauliSumXZ
from .sqd import cache_mode, subspace_states, unpack_states

STATE_BITS = L.BATCH_STATE_BITS
_MODES = {'free': L.MODE_FREE, 'conn': L.MODE_CONN}


def composite_keys(states_list):
    """(keys, prow): keys (p << 40) | s of every problem's sorted states, prow[p] = first row."""
    counts = np.array([len(s) for s in states_list], dtype=np.int64)
    prow = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    keys = np.empty(int(prow[-1]), dtype=np.uint64)
    for p, s in enumerate(states_list):
        s = np.asarray(s, dtype=np.uint64)
        if len(s) and int(s[-1]) >> STATE_BITS:
            raise ValueError(f'problem {p}: states need at most {STATE_BITS} bits')
        keys[prow[p]:prow[p + 1]] = (np.uint64(p) << np.uint64(STATE_BITS)) | s
    return keys, prow


def concat_terms(hamiltonians):
    """Grouped terms of every problem concatenated: (xmask, toff, zmask, coef, gofs, dgrp,
    is_real); toff runs over all terms, dgrp[p] is the global index of problem p's x = 0 group
    or -1."""
    xs, zs, cs, tof, gofs, dgrp = [], [], [], [np.zeros(1, np.int64)], [0], []
    real = True
    nterm = 0
    for h in hamiltonians:
        xmask, toff, zmask, coef, dg, is_real = h.device_arrays(truncate=True)
        if len(xmask) and int(np.max(xmask)) >> STATE_BITS:
            raise ValueError(f'X masks need at most {STATE_BITS} bits')
        xs.append(xmask)
        zs.append(zmask)
        cs.append(coef)
        tof.append(toff[1:].astype(np.int64) + nterm)
        dgrp.append(gofs[-1] + dg if dg >= 0 else -1)
        gofs.append(gofs[-1] + len(xmask))
        nterm += len(zmask)
        real = real and is_real
    toff = np.concatenate(tof)
    if toff[-1] >= 2 ** 31:
        raise ValueError('too many terms for int32 offsets')
    return (np.concatenate(xs).astype(np.uint64), toff.astype(np.int32),
            np.concatenate(zs).astype(np.uint64), np.concatenate(cs).astype(np.complex128),
            np.asarray(gofs, np.int32), np.asarray(dgrp, np.int32), real)


class BatchedSQD:
    """P SQD problems in one device batch.

    ``hamiltonians``: list of ``PauliSumXZ`` (or anything ``PauliSumXZ.from_paulisum`` takes);
    ``states_list``: per problem a sorted distinct uint64 array or a (D, n) 0/1 array;
    ``cache_level``: (0, *) lookups in every matvec ('free'), (1, 0|1) cached source lists;
    ``states_sizes``: per problem the convergence length of ``sqd()``'s ``states_size``
    (default: the length of the states array given, as ``sqd()``).
    """

    def __init__(self, hamiltonians, states_list, cache_level=(0, 0), states_sizes=None,
                 filter=True, device=None, stream=None, presence=None, tune_cache=None,
                 line_filter=True, line_bits=8):
        """``cache_level='auto'``: matrix-free or cached connectivity, chosen by measurement
        (``rqutils_gb300.autotune.tune_batch``, recorded per problem class in ``tune_cache``).
        ``line_filter``: probe a line filter over the composite keys (2^line_bits-bit lines, each
        problem with its own prefix shift, two bits per row in one word) before the hash table
        instead of the presence bitmap (``presence``, used only without it): 11.6 against 12.6 ms
        per batched product on 256 random problems of up to 40 qubits."""
        if len(hamiltonians) != len(states_list) or not hamiltonians:
            raise ValueError('need one subspace per Hamiltonian and at least one problem')
        self.device = device or default_device()
        hams = [h if isinstance(h, PauliSumXZ)
                else PauliSumXZ.from_paulisum(h, force_real=True, add_padding=True)
                for h in hamiltonians]
        if cache_level == 'auto':
            from .autotune import tune_batch
            sl = [subspace_states(s, h.num_qubits) for h, s in zip(hams, states_list)]
            (mode, _, lb), _ = tune_batch(hams, sl, cache=tune_cache, device=self.device)
            cache_level = (0, 0) if mode == 'free' else (1, 0)
            line_filter = lb > 0
        for h in hams:
            if h.num_qubits > STATE_BITS:
                raise ValueError(f'batched problems have at most {STATE_BITS} qubits')
        self.hams = hams
        n_in = [np.asarray(s).shape[0] for s in states_list]
        self.states = [subspace_states(s, h.num_qubits) for h, s in zip(hams, states_list)]
        if any(len(s) == 0 for s in self.states):
            raise ValueError('empty subspace')
        sizes = n_in if states_sizes is None else [int(v) for v in states_sizes]
        if len(sizes) != len(hams) or any(a < b for a, b in zip(sizes, n_in)):
            raise ValueError('states_sizes: one per problem, not below its states array length')
        self.states_size = (ctypes.c_int64 * len(sizes))(*sizes)
        mode = cache_mode(cache_level)
        if mode not in _MODES:
            raise ValueError('batched problems support cache_level (0, *) and (1, 0|1)')
        self.mode = mode
        self.P = len(hams)
        keys, prow = composite_keys(self.states)
        self.prow = prow
        self.D = int(prow[-1])
        xmask, toff, zmask, coef, gofs, dgrp, real = concat_terms(hams)
        self.is_real = real
        self.gofs_host, self.dgrp_host = gofs, dgrp
        dev = self.device
        self.keys = _u64_tensor(keys, dev)
        self.prow_t = torch.from_numpy(prow).to(dev)
        self.xmask = _u64_tensor(xmask if len(xmask) else np.zeros(1, np.uint64), dev)
        self.toff = torch.from_numpy(toff).to(dev)
        self.zmask = _u64_tensor(zmask if len(zmask) else np.zeros(1, np.uint64), dev)
        cf = coef if len(coef) else np.zeros(1, np.complex128)
        self.coef = torch.from_numpy(np.ascontiguousarray(cf).view(np.float64)).to(dev)
        self.gofs = torch.from_numpy(gofs).to(dev)
        self.dgrp = torch.from_numpy(dgrp).to(dev)
        J = len(xmask)
        self.xhash = torch.empty(max(J, 1), dtype=torch.int32, device=dev)
        terms = L.Terms(J=J, K=len(zmask), diag_group=-1, is_real=int(real),
                        xmask=L.ptr(self.xmask), toff=L.ptr(self.toff), zmask=L.ptr(self.zmask),
                        coef=L.ptr(self.coef), xhash=None)
        lib = L.lib()
        if J:
            L.check(lib.rq_terms_hash(ctypes.byref(terms), L.ptr(self.xhash), L.stream_ptr(stream)),
                    'rq_terms_hash')
        terms.xhash = L.ptr(self.xhash)
        hb = ctypes.c_int32()
        L.check(lib.rq_subspace_sizes(self.D, 64, ctypes.byref(hb)), 'rq_subspace_sizes')
        self.hkeys = torch.empty(4 << hb.value, dtype=torch.int64, device=dev)
        self.hvals = torch.empty(4 << hb.value, dtype=torch.int32, device=dev)
        pb = ctypes.c_int32()
        L.check(lib.rq_presence_bits(self.D, 64, ctypes.byref(pb)), 'rq_presence_bits')
        self.pbits = pb.value if presence is None else (0 if presence is False else int(presence))
        if line_filter:
            self.pbits = 0
            lb = ctypes.c_int32()
            L.check(lib.rq_line_filter_bits(self.D, int(line_bits), ctypes.byref(lb)),
                    'rq_line_filter_bits')
            self.lbits, self.lwbits = lb.value, int(line_bits)
            self.lmap = torch.empty(1 << (self.lbits + self.lwbits - 5), dtype=torch.int32,
                                    device=dev)
            self.xline = torch.empty(max(J, 1), dtype=torch.int32, device=dev)
            self.lshift = torch.empty(self.P, dtype=torch.int32, device=dev)
        else:
            self.lbits = self.lwbits = 0
            self.lmap = self.xline = self.lshift = None
        self.pmap = (torch.empty((1 << self.pbits) // 32, dtype=torch.int32, device=dev)
                     if self.pbits else None)
        if filter:
            fm = np.array([default_filter_masks(h.num_qubits) for h in hams],
                          dtype=np.uint64).reshape(-1)
            self.fmask = _u64_tensor(fm, dev)
        else:
            self.fmask = None
        self.fbits = torch.empty(self.P * L.FILTER_WORDS, dtype=torch.int32, device=dev)
        self.diag0 = torch.empty(self.D, dtype=torch.float64, device=dev)
        self.scratch = scratch_tensor(self.D, dev)
        self.c = L.Batch(P=self.P, mode=L.MODE_FREE, keys=L.ptr(self.keys),
                         prow=L.ptr(self.prow_t), D=self.D, hkeys=L.ptr(self.hkeys),
                         hvals=L.ptr(self.hvals), hbits=hb.value, pbits=self.pbits, empty_key=0,
                         fmask=L.ptr(self.fmask), fbits=L.ptr(self.fbits), terms=terms,
                         gofs=L.ptr(self.gofs), dgrp=L.ptr(self.dgrp), diag0=L.ptr(self.diag0),
                         states_size=ctypes.cast(self.states_size, ctypes.c_void_p),
                         pmap=L.ptr(self.pmap), lmap=L.ptr(self.lmap), xline=L.ptr(self.xline),
                         lshift=L.ptr(self.lshift), lbits=self.lbits, lwbits=self.lwbits)
        L.check(lib.rq_batch_build(ctypes.byref(self.c), L.ptr(self.scratch), L.stream_ptr(stream)),
                'rq_batch_build')
        self.rowptr = self.col = self.grp = None
        self.nnz = 0
        if mode == 'conn':
            self._build_conn(stream)
        self.c.mode = _MODES[mode]
        self.dtype = torch.float64 if real else torch.complex128

    def _build_conn(self, stream=None):
        lib = L.lib()
        self.rowptr = torch.empty(self.D + 1, dtype=torch.int64, device=self.device)
        nnz = ctypes.c_int64()
        L.check(lib.rq_batch_conn_build(ctypes.byref(self.c), L.ptr(self.rowptr), None, None,
                                        ctypes.byref(nnz), L.ptr(self.scratch),
                                        L.stream_ptr(stream)), 'rq_batch_conn_build (count)')
        self.nnz = int(nnz.value)
        n = max(self.nnz, 1)
        self.col = torch.empty(n, dtype=torch.int32, device=self.device)
        self.grp = torch.empty(n, dtype=torch.int32, device=self.device)
        L.check(lib.rq_batch_conn_build(ctypes.byref(self.c), L.ptr(self.rowptr), L.ptr(self.col),
                                        L.ptr(self.grp), ctypes.byref(nnz), L.ptr(self.scratch),
                                        L.stream_ptr(stream)), 'rq_batch_conn_build (fill)')
        self.c.rowptr, self.c.col, self.c.grp = L.ptr(self.rowptr), L.ptr(self.col), L.ptr(self.grp)
        self.c.nnz = self.nnz

    # ------------------------------------------------------------------------------------------
    def rows(self, p):
        return slice(int(self.prow[p]), int(self.prow[p + 1]))

    def split(self, x):
        """Per-problem views of a batch vector."""
        return [x[self.rows(p)] for p in range(self.P)]

    def matvec(self, x, out=None, stream=None):
        """y_p = H_p x_p for every problem (one launch)."""
        vt = VTYPE_OF.get(x.dtype)
        if vt is None:
            raise TypeError(f'unsupported dtype {x.dtype}')
        x = x.contiguous()
        if out is None:
            out = torch.empty_like(x)
        L.check(L.lib().rq_batch_matvec(ctypes.byref(self.c), vt, L.ptr(x), L.ptr(out),
                                        L.ptr(self.scratch), L.stream_ptr(stream)),
                'rq_batch_matvec')
        return out

    __call__ = matvec

    def check_errors(self):
        flag = int(self.scratch[16:20].view(torch.int32).item())
        if flag:
            raise L.RqError(flag, 'a batched matvec kernel reported an error')

    def initial_vectors(self, dtype=None):
        """sqd.py:373-398 per problem: one-hot at the first minimum of the x = 0 diagonal when
        that group is the problem's first group, else at the problem's first row."""
        dtype = dtype or self.dtype
        x0 = torch.zeros(self.D, dtype=dtype, device=self.device)
        d = self.diag0.cpu().numpy()
        starts = self.prow[:-1]
        counts = np.diff(self.prow)
        mins = np.minimum.reduceat(d, starts)
        hit = np.flatnonzero(d == np.repeat(mins, counts))
        first = hit[np.searchsorted(hit, starts)]
        use_diag = self.dgrp_host == self.gofs_host[:-1]
        idx = np.where(use_diag, first, starts)
        x0[torch.from_numpy(idx.astype(np.int64)).to(self.device)] = 1
        return x0

    def solve(self, x0=None, maxiter=1000, tol=None, variant='reference', precision='fp64',
              target_rel=None, switch_rel=1e-5, refresh=32, use_graph=True, jacobi=False,
              guard=True, stream=None):
        """LOBPCG on every problem (rq_batch_solve).  ``precision``: 'fp64' (float64 /
        complex128), 'fp32' (float32 / complex64 vectors, FP64 reductions) or 'mixed' (a 32-bit
        phase, then FP64).  Returns (eigvals (P,), x (D,), [info per problem])."""
        if x0 is None:
            vt = vtype_for(self.is_real, 'fp32' if precision == 'fp32' else 'fp64')
            x0 = self.initial_vectors(TORCH_DTYPE[vt])
        x0 = x0.contiguous()
        vt = VTYPE_OF[x0.dtype]
        prm = _params(0, vt, maxiter, tol, 0, variant, precision == 'mixed', target_rel,
                      switch_rel, refresh, use_graph, jacobi, guard)
        n = ctypes.c_size_t()
        lib = L.lib()
        L.check(lib.rq_batch_workspace_size(ctypes.byref(self.c), ctypes.byref(prm),
                                            ctypes.byref(n)), 'rq_batch_workspace_size')
        ws = getattr(self, '_ws', None)
        if ws is None or ws.numel() < n.value:
            ws = self._ws = torch.empty(int(n.value), dtype=torch.uint8, device=self.device)
        xout = torch.empty_like(x0)
        res = (L.LobpcgResult * self.P)()
        L.check(lib.rq_batch_solve(ctypes.byref(self.c), ctypes.byref(prm), L.ptr(ws), L.ptr(x0),
                                   L.ptr(xout), res, L.stream_ptr(stream)), 'rq_batch_solve')
        self.check_errors()
        infos = [_info(r) for r in res]
        return np.array([r.eigval for r in res]), xout, infos


def sqd_batch(hamiltonians, states_list, states_sizes=None, return_eigvec=True,
              cache_level=(1, 0), *, precision='fp64', variant='reference', maxiter=1000,
              tol=None, target_rel=None, jacobi=False, use_graph=True, return_info=False,
              device=None):
    """``sqd()`` on many problems at once: a list of energies, or of
    ``(energy, eigvec, basis_states)`` per problem with ``return_eigvec``."""
    b = BatchedSQD(hamiltonians, states_list, cache_level=cache_level, states_sizes=states_sizes,
                   device=device)
    eig, x, infos = b.solve(maxiter=maxiter, tol=tol, variant=variant, precision=precision,
                            target_rel=target_rel, use_graph=use_graph, jacobi=jacobi)
    if not return_eigvec:
        out = [float(e) for e in eig]
    else:
        xs = x.cpu().numpy()
        out = [(float(eig[p]), xs[b.rows(p)], unpack_states(b.states[p], b.hams[p].num_qubits))
               for p in range(b.P)]
    return (out, infos) if return_info else out
