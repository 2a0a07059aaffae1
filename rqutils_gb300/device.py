"""Device-resident SQD objects over the C ABI.

* ``DeviceSubspace``  -- sorted uint64 states in HBM, the bucketed hash table (or the sampled
  binary-search form) and the sector filter (``rq_subspace_build``).
* ``DeviceTerms``     -- a ``PauliSumXZ`` in the grouped device layout (``rq_terms_t``).
* ``DeviceOperator``  -- terms on a subspace with a matvec mode (the reference's ``cache_level``):
  ``free`` (lookups in every matvec), ``conn`` (cached source lists, diagonals recomputed) or
  ``csr`` (cached matrix elements); the x = 0 group's diagonal is cached in FP64.

Buffers are torch tensors (PyTorch is used for device memory and streams only); every computation
is a call into librqsqd.so.  uint64 data is stored in int64 tensors (same bits).
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from .paulis.symplectic import PauliSumXZ

TORCH_DTYPE = {L.F32: torch.float32, L.F64: torch.float64, L.C64: torch.complex64,
               L.C128: torch.complex128}
VTYPE_OF = {v: k for k, v in TORCH_DTYPE.items()}


def default_device():
    if not torch.cuda.is_available():
        raise RuntimeError('rqutils_gb300 needs a CUDA device (there is no CPU fallback)')
    return torch.device('cuda', torch.cuda.current_device())


def _u64_tensor(a, device):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.uint64))
    return torch.from_numpy(a.view(np.int64)).to(device)


def vtype_for(real, precision='fp64'):
    """Value type code: real/complex x 32/64-bit."""
    if precision in ('fp32', 'single', '32'):
        return L.F32 if real else L.C64
    return L.F64 if real else L.C128


def scratch_tensor(D, device):
    n = ctypes.c_size_t()
    L.check(L.lib().rq_scratch_size(int(D), ctypes.byref(n)), 'rq_scratch_size')
    return torch.zeros(int(n.value), dtype=torch.uint8, device=device)


def default_filter_masks(n):
    """Sector filter split: qubits [0, n/2) and [n/2, n) (the spin halves of a JW ordering with
    all up orbitals first; for a fixed-weight subspace any split rejects weight changes)."""
    if n <= 1:
        return 0, 0
    half = n // 2
    a = (1 << half) - 1
    b = ((1 << n) - 1) ^ a if n < 64 else (0xFFFFFFFFFFFFFFFF ^ a)
    return a, b


class DeviceSubspace:
    """Sorted distinct states (uint64, bit q = qubit q) with their lookup structures."""

    def __init__(self, states, num_qubits=64, lookup='hash', filter_masks=None, device=None,
                 stream=None, key_bits=None, presence=None, line_filter=True, line_bits=8):
        """``presence``: None = a presence bitmap when the hash table does not fit in L2
        (rq_presence_bits), False = none, an int = its size log2.  ``line_filter``: build the
        line filter (lines of 2^line_bits bits, 8..10) that the matrix-free kernel probes before
        the key buckets (same results; False probes the key buckets directly)."""
        self.device = device or default_device()
        if isinstance(states, torch.Tensor):
            self.states = states.to(self.device, dtype=torch.int64).contiguous()
        else:
            self.states = _u64_tensor(states, self.device)
        self.D = int(self.states.numel())
        if self.D < 1:
            raise ValueError('empty subspace')
        self.num_qubits = num_qubits
        self.lookup = {'hash': L.LOOKUP_HASH, 'bsearch': L.LOOKUP_BSEARCH}[lookup]
        # 32-bit keys when every state and X mask fits (num_qubits <= 32): 8 keys per bucket
        if key_bits is None:
            key_bits = 32 if num_qubits <= 32 else 64
        if key_bits == 32 and num_qubits > 32:
            raise ValueError('32-bit keys need num_qubits <= 32')
        self.key_bits = key_bits
        hb = ctypes.c_int32()
        L.check(L.lib().rq_subspace_sizes(self.D, key_bits, ctypes.byref(hb)), 'rq_subspace_sizes')
        self.hbits = hb.value
        if self.lookup == L.LOOKUP_HASH:
            # 2^hbits buckets of 4 keys (16 or 32 bytes)
            self.hkeys = torch.empty((4 * key_bits // 64) << self.hbits, dtype=torch.int64,
                                     device=self.device)
            self.hvals = torch.empty(4 << self.hbits, dtype=torch.int32, device=self.device)
        else:
            self.hkeys = self.hvals = None
        self.lmap, self.lbits, self.lwbits = None, 0, 0
        if self.lookup == L.LOOKUP_HASH and line_filter:
            lb = ctypes.c_int32()
            L.check(L.lib().rq_line_filter_bits(self.D, int(line_bits), ctypes.byref(lb)),
                    'rq_line_filter_bits')
            self.lbits, self.lwbits = lb.value, int(line_bits)
            self.lmap = torch.empty(1 << (self.lbits + self.lwbits - 5), dtype=torch.int32,
                                    device=self.device)
        self.fbits = torch.zeros(L.FILTER_WORDS, dtype=torch.int32, device=self.device)
        # presence bitmap in front of a hash table too large for L2
        self.pbits = 0
        self.pmap = None
        if self.lookup == L.LOOKUP_HASH and presence is not False:
            pb = ctypes.c_int32()
            L.check(L.lib().rq_presence_bits(self.D, key_bits, ctypes.byref(pb)),
                    'rq_presence_bits')
            self.pbits = pb.value if presence is None else int(presence)
            if self.pbits:
                self.pmap = torch.empty((1 << self.pbits) // 32, dtype=torch.int32,
                                        device=self.device)
        fa, fb = filter_masks if filter_masks is not None else default_filter_masks(num_qubits)
        self.scratch = scratch_tensor(self.D, self.device)
        self.c = L.Subspace(states=L.ptr(self.states), D=self.D, hkeys=L.ptr(self.hkeys),
                            hvals=L.ptr(self.hvals), hbits=self.hbits, lookup=self.lookup,
                            key_bits=key_bits, pbits=self.pbits, empty_key=0, fmask_a=int(fa),
                            fmask_b=int(fb), fbits=L.ptr(self.fbits), pmap=L.ptr(self.pmap),
                            lmap=L.ptr(self.lmap), lbits=self.lbits, lwbits=self.lwbits,
                            lshift=0, fpoint=-1)
        L.check(L.lib().rq_subspace_build(ctypes.byref(self.c), L.ptr(self.scratch),
                                          L.stream_ptr(stream)), 'rq_subspace_build')

    def states_numpy(self):
        return self.states.cpu().numpy().view(np.uint64)

    def xsource(self, xmasks, stream=None):
        """get_xsource for each X mask: (J, D) int32 on the device (-1 = not in the subspace)."""
        xm = _u64_tensor(np.atleast_1d(xmasks), self.device)
        out = torch.empty((xm.numel(), self.D), dtype=torch.int32, device=self.device)
        L.check(L.lib().rq_xsource(ctypes.byref(self.c), L.ptr(xm), int(xm.numel()), L.ptr(out),
                                   L.stream_ptr(stream)), 'rq_xsource')
        return out


class DeviceTerms:
    """A PauliSumXZ in the C ABI's grouped layout."""

    def __init__(self, ham: PauliSumXZ, device=None, truncate=True):
        self.device = device or default_device()
        xmask, toff, zmask, coef, diag_group, is_real = ham.device_arrays(truncate=truncate)
        self.J, self.K = len(xmask), len(zmask)
        self.diag_group = diag_group
        self.is_real = is_real
        self.num_qubits = ham.num_qubits
        dev = self.device
        self.xmask = torch.empty(max(self.J, 1), dtype=torch.int64, device=dev)
        self.toff = torch.empty(self.J + 1, dtype=torch.int32, device=dev)
        self.zmask = torch.empty(max(self.K, 1), dtype=torch.int64, device=dev)
        self.coef = torch.empty(2 * max(self.K, 1), dtype=torch.float64, device=dev)
        self.xhash = torch.empty(max(self.J, 1), dtype=torch.int32, device=dev)
        self.group_sizes = np.diff(toff)
        xh = np.ascontiguousarray(xmask, dtype=np.uint64)
        th = np.ascontiguousarray(toff, dtype=np.int32)
        zh = np.ascontiguousarray(zmask, dtype=np.uint64)
        ch = np.ascontiguousarray(coef, dtype=np.complex128)
        self.c = L.Terms()
        L.check(L.lib().rq_terms_upload(self.J, self.K, xh.ctypes.data, th.ctypes.data,
                                        zh.ctypes.data, ch.ctypes.data, L.ptr(self.xmask),
                                        L.ptr(self.toff), L.ptr(self.zmask), L.ptr(self.coef),
                                        L.ptr(self.xhash), ctypes.byref(self.c), L.stream_ptr()),
                'rq_terms_upload')
        # the dtype rule of the reference (every phased coefficient real) over all terms
        self.c.is_real = int(is_real)


class DeviceOperator:
    """H restricted to a DeviceSubspace.  mode: 'free' | 'conn' | 'csr'."""

    MODES = {'free': L.MODE_FREE, 'conn': L.MODE_CONN, 'csr': L.MODE_CSR}

    def __init__(self, terms: DeviceTerms, subspace: DeviceSubspace, mode='conn', cache_diag=True,
                 csr_vtype=None, stream=None):
        if terms.device != subspace.device:
            raise ValueError('terms and subspace live on different devices')
        self.terms, self.sub = terms, subspace
        self.device = subspace.device
        self.D = subspace.D
        self.mode = mode
        self.is_real = terms.is_real
        self.scratch = scratch_tensor(self.D, self.device)
        self.diag0 = None
        if terms.diag_group >= 0 and (cache_diag or mode == 'csr'):
            self.diag0 = self.group_diagonal(terms.diag_group, stream=stream).real.contiguous()
        self.rowptr = self.col = self.grp = self.val = None
        self.nnz = 0
        self.csr_vtype = None
        self.c = L.Operator(sub=subspace.c, terms=terms.c, mode=L.MODE_FREE,
                            diag0=L.ptr(self.diag0))
        if mode in ('conn', 'csr'):
            self._build_conn(with_values=(mode == 'csr'),
                             vtype=csr_vtype if csr_vtype is not None
                             else vtype_for(self.is_real), stream=stream)
        self.c.mode = self.MODES[mode]

    # ------------------------------------------------------------------------------------------
    def group_diagonal(self, g, stream=None):
        """get_diagonal of group g on the subspace: complex128 (D,)."""
        a, b = int(self.terms.toff[g]), int(self.terms.toff[g + 1])
        out = torch.empty(self.D, dtype=torch.complex128, device=self.device)
        zm = self.terms.zmask[a:b] if b > a else self.terms.zmask[:1]
        cf = self.terms.coef[2 * a:2 * b] if b > a else self.terms.coef[:2]
        L.check(L.lib().rq_diagonal(L.ptr(self.sub.states), self.D, L.ptr(zm), L.ptr(cf), b - a,
                                    L.ptr(out), L.stream_ptr(stream)), 'rq_diagonal')
        return out

    def _build_conn(self, with_values, vtype, stream=None):
        lib = L.lib()
        self.rowptr = torch.empty(self.D + 1, dtype=torch.int64, device=self.device)
        nnz = ctypes.c_int64()
        L.check(lib.rq_conn_build(ctypes.byref(self.c), L.ptr(self.rowptr), None, None, None, vtype,
                                  ctypes.byref(nnz), L.ptr(self.scratch), L.stream_ptr(stream)),
                'rq_conn_build (count)')
        self.nnz = int(nnz.value)
        n = max(self.nnz, 1)
        self.col = torch.empty(n, dtype=torch.int32, device=self.device)
        self.grp = torch.empty(n, dtype=torch.int32, device=self.device)
        if with_values:
            self.val = torch.empty(n, dtype=TORCH_DTYPE[vtype], device=self.device)
            self.csr_vtype = vtype
            self.c.val_vtype = vtype
        L.check(lib.rq_conn_build(ctypes.byref(self.c), L.ptr(self.rowptr), L.ptr(self.col),
                                  L.ptr(self.grp), L.ptr(self.val), vtype, ctypes.byref(nnz),
                                  L.ptr(self.scratch), L.stream_ptr(stream)), 'rq_conn_build (fill)')
        self.c.rowptr = L.ptr(self.rowptr)
        self.c.col = L.ptr(self.col)
        self.c.grp = L.ptr(self.grp)
        self.c.val = L.ptr(self.val)
        self.c.nnz = self.nnz

    # ------------------------------------------------------------------------------------------
    def matvec(self, x, out=None, stream=None):
        """y = H x for a device tensor x of dtype float32/64 or complex64/128."""
        vt = VTYPE_OF.get(x.dtype)
        if vt is None:
            raise TypeError(f'unsupported dtype {x.dtype}')
        x = x.contiguous()
        if out is None:
            out = torch.empty_like(x)
        L.check(L.lib().rq_matvec(ctypes.byref(self.c), vt, L.ptr(x), L.ptr(out),
                                  L.ptr(self.scratch), L.stream_ptr(stream)), 'rq_matvec')
        return out

    __call__ = matvec

    def check_errors(self):
        """Raise if a kernel flagged an error (the flag lives 16 bytes into the scratch)."""
        flag = int(self.scratch[16:20].view(torch.int32).item())
        if flag:
            raise L.RqError(flag, 'a matvec kernel reported an error')

    def connectivity(self):
        """(rowptr, col, grp) on the host (conn/csr modes)."""
        if self.rowptr is None:
            raise RuntimeError('connectivity is cached only in conn/csr modes')
        return (self.rowptr.cpu().numpy(), self.col[:self.nnz].cpu().numpy(),
                self.grp[:self.nnz].cpu().numpy())


def fullspace_matmul(ham: PauliSumXZ, rhs):
    """PauliSumXZ.matmul on the GPU (rq_fullspace_matvec), column by column for 2-d rhs."""
    device = default_device()
    as_numpy = not isinstance(rhs, torch.Tensor)
    r = torch.as_tensor(np.asarray(rhs)) if as_numpy else rhs
    n = ham.num_qubits
    terms = DeviceTerms(ham, device=device, truncate=False)
    real = terms.is_real and not torch.is_complex(r)
    vt = L.F64 if real else L.C128
    rd = r.to(device=device, dtype=TORCH_DTYPE[vt])
    cols = rd.reshape(rd.shape[0], -1)
    out = torch.empty_like(cols)
    for k in range(cols.shape[1]):
        xin = cols[:, k].contiguous()
        y = torch.empty_like(xin)
        L.check(L.lib().rq_fullspace_matvec(ctypes.byref(terms.c), n, vt, L.ptr(xin), L.ptr(y),
                                            L.stream_ptr()), 'rq_fullspace_matvec')
        out[:, k] = y
    out = out.reshape(rd.shape)
    return out.cpu().numpy() if as_numpy else out
