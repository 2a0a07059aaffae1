"""rq_lobpcg_solve_noalloc: the solve for callers that cannot allocate device memory.

Such callers -- a custom-call handler inside another framework, handed only its operand and result
buffers, or a service that reserved its device memory at start-up -- pass only their inputs and
outputs; the solver's workspace is a static device array of the library.  This file is collected
last so that a run stopping at the first failure has already run every other test; it also passes
on its own in a fresh process.
"""
import ctypes
import warnings

import numpy as np
import pytest

from golden_cases import load, hamiltonian

pytestmark = pytest.mark.gpu

EIG_RTOL = 1e-10


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _operator(name, cache_level=(1, 0)):
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import SQDProblem, subspace_states
    case = load(name)
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        h = PauliSumXZ.from_paulisum(hamiltonian(case), force_real=True, add_padding=True)
    S = subspace_states(case['states'], h.num_qubits)
    return SQDProblem(h, S, cache_level=cache_level)


def _solve_workspace(op, x0, prm):
    """The existing entry point, with a workspace allocated by the caller."""
    import torch
    from rqutils_gb300 import _lib as L
    lib = L.lib()
    n = ctypes.c_size_t()
    L.check(lib.rq_lobpcg_workspace_size(op.D, ctypes.byref(prm), ctypes.byref(n)))
    ws = torch.empty(n.value, dtype=torch.uint8, device=x0.device)
    xo = torch.empty_like(x0)
    res = L.LobpcgResult()
    L.check(lib.rq_lobpcg_solve(ctypes.byref(op.c), ctypes.byref(prm), L.ptr(ws), L.ptr(x0),
                                L.ptr(xo), ctypes.byref(res), L.stream_ptr()))
    return res, xo


def _solve_noalloc(op, x0, prm):
    import torch
    from rqutils_gb300 import _lib as L
    xo = torch.empty_like(x0)
    res = L.LobpcgResult()
    L.check(L.lib().rq_lobpcg_solve_noalloc(ctypes.byref(op.c), ctypes.byref(prm), L.ptr(x0),
                                            L.ptr(xo), ctypes.byref(res), L.stream_ptr()),
            'rq_lobpcg_solve_noalloc')
    return res, xo


@pytest.mark.parametrize('name,mixed,cache_level', [('local12', 0, (1, 0)), ('hubbard2x2', 0, (1, 0)),
                                                   ('n16dense', 1, (1, 0)), ('hubbard2x2', 1, (0, 0))])
def test_noalloc_matches_workspace_solve(name, mixed, cache_level):
    """Cached connectivity runs the persistent kernel in both calls; the matrix-free operator runs
    eager launches in the allocation-free call and CUDA-graph chunks in the workspace call."""
    import torch
    from rqutils_gb300 import _lib as L
    prob = _operator(name, cache_level)
    x0 = prob.initial_vector()
    vt = L.F64 if prob.terms.is_real else L.C128
    prm = L.LobpcgParams(maxiter=1000, variant=L.LOBPCG_REFERENCE, vtype=vt, mixed=mixed,
                         use_graph=1)
    ref, xref = _solve_workspace(prob.op, x0, prm)
    assert ref.converged
    for _ in range(2):  # two calls in a row share the static workspace
        res, xo = _solve_noalloc(prob.op, x0, prm)
        torch.cuda.synchronize()
        assert res.converged and res.status == L.OK
        assert abs(res.eigval - ref.eigval) <= EIG_RTOL * max(1.0, abs(ref.eigval))
        assert res.niter == ref.niter
        overlap = abs(torch.vdot(xref, xo).item())
        assert overlap > 1 - 1e-9


def test_noalloc_rejects_oversized_problem():
    from rqutils_gb300 import _lib as L
    op = L.Operator()
    op.sub.D = 1 << 20          # 2^20 rows of complex128 need far more than 8 MiB
    prm = L.LobpcgParams(maxiter=10, variant=L.LOBPCG_REFERENCE, vtype=L.C128)
    res = L.LobpcgResult()
    rc = L.lib().rq_lobpcg_solve_noalloc(ctypes.byref(op), ctypes.byref(prm), 1, 1,
                                         ctypes.byref(res), None)
    assert rc == L.E_RANGE
    assert b'static workspace holds' in L.lib().rq_last_error()


def test_noalloc_leaves_device_free_memory_unchanged():
    """The call allocates nothing: once a first call on the device has loaded the solver's kernels
    and looked up the static array's address, a further call leaves the device's free memory
    (cudaMemGetInfo) exactly as it was."""
    import torch
    from rqutils_gb300 import _lib as L
    prob = _operator('hubbard2x2')
    x0 = prob.initial_vector()
    vt = L.F64 if prob.terms.is_real else L.C128
    prm = L.LobpcgParams(maxiter=1000, variant=L.LOBPCG_REFERENCE, vtype=vt, use_graph=1)
    first, _ = _solve_noalloc(prob.op, x0, prm)
    xo = torch.empty_like(x0)
    res = L.LobpcgResult()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    rc = L.lib().rq_lobpcg_solve_noalloc(ctypes.byref(prob.op.c), ctypes.byref(prm), L.ptr(x0),
                                         L.ptr(xo), ctypes.byref(res), L.stream_ptr())
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert rc == L.OK and res.converged
    assert res.eigval == first.eigval
    assert free_after == free_before, free_before - free_after
