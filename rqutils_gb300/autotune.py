"""Measured choice of the matvec form -- the reference's ``cache_level``, made by timing.

The product y = H x on a sampled subspace has several forms here, and which is fastest depends on
the problem: the matrix-free hash lookup with a line filter of 256, 512 or 1024-bit lines or
without one, the matrix-free sampled binary search, the cached connectivity (one source row and
group per connection, diagonals recomputed) and the cached matrix elements.  The cached forms cost
a build and memory; the matrix-free ones cost more per product.

``tune(hamiltonian, states)`` builds every candidate that fits the memory budget, times the build
and the product (CUDA events on the current stream, the median of ``reps`` products after
``warmup``) and returns the candidate with the least ``build + expected_products * product``.
Choices are kept per problem class -- qubits, key width, log2 of the row count, log2 of the X-group
count and the vector type -- in a ``TuneCache`` (in memory, and in a JSON file when the cache has
a path), so a later problem of the class takes the recorded form without measuring.

``SQDProblem`` / ``sqd`` and ``BatchedSQD`` accept ``cache_level='auto'``, which uses this module
(for batches the candidates are the matrix-free form with the line filter or the presence
bitmap, and the cached-connectivity form).
"""
import json
import math
import os
import statistics
import threading
import time

import numpy as np

# forms: (mode, lookup, line_bits); line_bits 0 = no line filter
FORMS = (('free', 'hash', 8), ('free', 'hash', 9), ('free', 'hash', 10), ('free', 'hash', 0),
         ('free', 'bsearch', 0), ('conn', 'hash', 8), ('csr', 'hash', 8))

# bytes per cached connection: source row and group (int32 each), plus the element value of the
# CSR form at the vector type
_CONN_BYTES = 8


def form_key(form):
    mode, lookup, lb = form
    return f'{mode}/{lookup}/{lb}'


def form_of(key):
    mode, lookup, lb = key.split('/')
    return mode, lookup, int(lb)


def problem_class(kind, num_qubits, D, J, dtype):
    """The key under which a choice is recorded: problems of one class share it."""
    key_bits = 32 if num_qubits <= 32 else 64
    return (f'{kind}:n{int(num_qubits)}:k{key_bits}:d{int(round(math.log2(max(D, 1))))}'
            f':j{int(round(math.log2(max(J, 1))))}:{str(dtype).replace("torch.", "")}')


class TuneCache:
    """Recorded choices {problem class: {'form': key, 'times': {form key: seconds}}}.  With a
    path the records are read from and written back to that JSON file."""

    def __init__(self, path=None):
        self.path = path
        self._lock = threading.Lock()
        self.records = {}
        if path and os.path.exists(path):
            with open(path) as fh:
                self.records = json.load(fh)

    def get(self, cls):
        with self._lock:
            rec = self.records.get(cls)
        return form_of(rec['form']) if rec else None

    def put(self, cls, form, times):
        with self._lock:
            self.records[cls] = {'form': form_key(form),
                                 'times': {form_key(f): t for f, t in times.items()}}
            if self.path:
                tmp = self.path + '.tmp'
                with open(tmp, 'w') as fh:
                    json.dump(self.records, fh, indent=1, sort_keys=True)
                os.replace(tmp, self.path)


_DEFAULT = TuneCache()


def default_cache():
    return _DEFAULT


def _time_products(matvec, x, warmup, reps):
    import torch
    y = matvec(x)
    for _ in range(warmup):
        matvec(x, out=y)
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        matvec(x, out=y)
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    return statistics.median(ts)


def _bytes_per_value(dtype):
    import torch
    return torch.empty((), dtype=dtype).element_size()


def tune(hamiltonian, states, dtype=None, expected_products=400, warmup=2, reps=5,
         memory_budget=None, cache=None, device=None, forms=FORMS):
    """Fastest form for one problem.  ``hamiltonian`` a PauliSumXZ, ``states`` sorted distinct
    uint64 (host array or device tensor).  Returns (form, {form: seconds}); the seconds are
    build + expected_products x product.  A recorded choice of the problem class is returned
    without measuring (and with an empty table)."""
    import torch
    from .device import (DeviceOperator, DeviceSubspace, DeviceTerms, default_device,
                         vtype_for)
    dev = device or default_device()
    cache = cache if cache is not None else _DEFAULT
    n = hamiltonian.num_qubits
    D = int(states.numel() if isinstance(states, torch.Tensor) else len(states))
    J = len(hamiltonian.xmask)
    terms = DeviceTerms(hamiltonian, device=dev)
    if dtype is None:
        dtype = torch.float64 if terms.is_real else torch.complex128
    cls = problem_class('one', n, D, J, dtype)
    hit = cache.get(cls)
    if hit is not None:
        return hit, {}
    if memory_budget is None:
        free, _ = torch.cuda.mem_get_info(dev)
        memory_budget = free // 4
    rng = np.random.default_rng(0)
    xr = rng.normal(size=D) + (0 if terms.is_real else 1j) * rng.normal(size=D)
    x = torch.as_tensor(xr).to(dev, dtype)
    times, nnz = {}, None
    subspaces = {}  # one subspace per (lookup, line bits), shared by the forms that use it
    for form in forms:
        mode, lookup, lb = form
        try:
            key = (lookup, lb)
            if key not in subspaces:
                subspaces[key] = DeviceSubspace(states, num_qubits=n, lookup=lookup, device=dev,
                                                line_filter=lb > 0, line_bits=lb or 8)
            sub = subspaces[key]
            per = _CONN_BYTES + (_bytes_per_value(dtype) if mode == 'csr' else 0)
            if mode != 'free' and (D * max(J - 1, 0) > 4e9 or
                                   (nnz is not None and nnz * per > memory_budget)):
                continue  # the connectivity count alone would take seconds, or does not fit
            csr_vtype = (vtype_for(terms.is_real, 'fp32' if dtype in (torch.float32,
                                                                      torch.complex64)
                                   else 'fp64') if mode == 'csr' else None)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()  # the operator's build (the subspace is common to all)
            op = DeviceOperator(terms, sub, mode=mode, csr_vtype=csr_vtype)
            torch.cuda.synchronize(dev)
            build = time.perf_counter() - t0
            if mode != 'free':
                nnz = op.nnz
                if nnz * per > memory_budget:
                    continue
            t = _time_products(op.matvec, x, warmup, reps)
            times[form] = build + expected_products * t
        except (RuntimeError, MemoryError):  # a form that does not fit: not a candidate
            torch.cuda.empty_cache()
            continue
    if not times:
        raise RuntimeError('autotune: no matvec form could be built')
    best = min(times, key=times.get)
    cache.put(cls, best, times)
    return best, times


def tune_batch(hamiltonians, states_list, dtype=None, expected_products=400, warmup=2, reps=5,
               cache=None, device=None):
    """Matrix-free (with the line filter or the presence bitmap in front of the table) or cached
    connectivity for a batch (BatchedSQD): the same measurement over the batch's forms
    (``hamiltonians`` PauliSumXZ, ``states_list`` sorted uint64 arrays).  Returns
    ('free' | 'conn', {form: seconds}); the line-filter choice is in the form's line bits
    (8 = line filter, 0 = presence bitmap)."""
    import torch
    from .batch import BatchedSQD
    cache = cache if cache is not None else _DEFAULT
    D = sum(len(s) for s in states_list)
    n = max(h.num_qubits for h in hamiltonians)
    J = sum(len(h.xmask) for h in hamiltonians)
    real = all(h.is_real for h in hamiltonians)
    dt = dtype or (torch.float64 if real else torch.complex128)
    cls = problem_class('batch', n, D, J, dt)
    hit = cache.get(cls)
    if hit is not None:
        return hit, {}
    rng = np.random.default_rng(0)
    times = {}
    for mode, cl, lb in (('free', (0, 0), 8), ('free', (0, 0), 0), ('conn', (1, 0), 8)):
        try:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b = BatchedSQD(hamiltonians, states_list, cache_level=cl, device=device,
                           line_filter=lb > 0, line_bits=lb or 8)
            torch.cuda.synchronize()
            build = time.perf_counter() - t0
        except (RuntimeError, MemoryError):  # a form that does not fit: not a candidate
            torch.cuda.empty_cache()
            continue
        xr = rng.normal(size=b.D) + (0 if real else 1j) * rng.normal(size=b.D)
        probe = torch.as_tensor(xr).to(b.device, dt)
        times[(mode, 'hash', lb)] = build + expected_products * _time_products(
            b.matvec, probe, warmup, reps)
        del b
    if not times:
        raise RuntimeError('autotune: no batched form could be built')
    best = min(times, key=times.get)
    cache.put(cls, best, times)
    return best, times
