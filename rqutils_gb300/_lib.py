"""ctypes binding of the C ABI declared in include/rqsqd.h (librqsqd.so).

This module is the whole Python <-> CUDA boundary: every device computation of the package is a
call through these functions.  There is no fallback: if the shared library is missing or cannot
be loaded, ``lib()`` raises and so does every operation that needs it.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'librqsqd.so')

F32, F64, C64, C128 = 0, 1, 2, 3
OK, E_ARG, E_CUDA, E_UNSORTED, E_TABLE, E_NONFINITE, E_MAXITER, E_RANGE = range(8)
LOOKUP_HASH, LOOKUP_BSEARCH, LOOKUP_IDENTITY = 0, 1, 2
MODE_FREE, MODE_CONN, MODE_CSR = 0, 1, 2
LOBPCG_REFERENCE, LOBPCG_FAST = 0, 1
FILTER_WORDS = 133

_c_void_p = ctypes.c_void_p


class Subspace(ctypes.Structure):
    _fields_ = [('states', _c_void_p), ('D', ctypes.c_int64), ('hkeys', _c_void_p),
                ('hvals', _c_void_p), ('hbits', ctypes.c_int32), ('lookup', ctypes.c_int32),
                ('key_bits', ctypes.c_int32), ('pbits', ctypes.c_int32),
                ('empty_key', ctypes.c_uint64), ('fmask_a', ctypes.c_uint64),
                ('fmask_b', ctypes.c_uint64), ('fbits', _c_void_p), ('pmap', _c_void_p),
                ('lmap', _c_void_p), ('lbits', ctypes.c_int32), ('lwbits', ctypes.c_int32),
                ('lshift', ctypes.c_int32), ('fpoint', ctypes.c_int32)]


class Terms(ctypes.Structure):
    _fields_ = [('J', ctypes.c_int32), ('K', ctypes.c_int32), ('diag_group', ctypes.c_int32),
                ('is_real', ctypes.c_int32), ('xmask', _c_void_p), ('toff', _c_void_p),
                ('zmask', _c_void_p), ('coef', _c_void_p), ('xhash', _c_void_p)]


class Operator(ctypes.Structure):
    _fields_ = [('sub', Subspace), ('terms', Terms), ('mode', ctypes.c_int32),
                ('val_vtype', ctypes.c_int32), ('diag0', _c_void_p), ('rowptr', _c_void_p),
                ('col', _c_void_p), ('grp', _c_void_p), ('val', _c_void_p),
                ('nnz', ctypes.c_int64)]


class LobpcgParams(ctypes.Structure):
    _fields_ = [('maxiter', ctypes.c_int32), ('variant', ctypes.c_int32),
                ('vtype', ctypes.c_int32), ('mixed', ctypes.c_int32), ('tol', ctypes.c_double),
                ('tol_dim', ctypes.c_double), ('switch_rel', ctypes.c_double),
                ('target_rel', ctypes.c_double), ('refresh', ctypes.c_int32),
                ('use_graph', ctypes.c_int32), ('jacobi', ctypes.c_int32),
                ('guard', ctypes.c_int32), ('restart', ctypes.c_int32), ('pad_', ctypes.c_int32)]


class LobpcgResult(ctypes.Structure):
    _fields_ = [('eigval', ctypes.c_double), ('resnorm', ctypes.c_double),
                ('axnorm', ctypes.c_double), ('niter', ctypes.c_int32),
                ('niter_lo', ctypes.c_int32), ('matvecs', ctypes.c_int32),
                ('converged', ctypes.c_int32), ('status', ctypes.c_int32),
                ('pad_', ctypes.c_int32)]


class Batch(ctypes.Structure):
    _fields_ = [('P', ctypes.c_int32), ('mode', ctypes.c_int32), ('keys', _c_void_p),
                ('prow', _c_void_p), ('D', ctypes.c_int64), ('hkeys', _c_void_p),
                ('hvals', _c_void_p), ('hbits', ctypes.c_int32), ('pbits', ctypes.c_int32),
                ('empty_key', ctypes.c_uint64), ('fmask', _c_void_p), ('fbits', _c_void_p),
                ('terms', Terms), ('gofs', _c_void_p), ('dgrp', _c_void_p), ('diag0', _c_void_p),
                ('rowptr', _c_void_p), ('col', _c_void_p), ('grp', _c_void_p),
                ('nnz', ctypes.c_int64), ('states_size', _c_void_p), ('pmap', _c_void_p),
                ('lmap', _c_void_p), ('xline', _c_void_p), ('lshift', _c_void_p),
                ('lbits', ctypes.c_int32), ('lwbits', ctypes.c_int32)]


BATCH_STATE_BITS = 40
MLP_IN, MLP_HIDDEN, MLP_OUT = 64, 256, 2
MLP_NPARAMS = 256 * 64 + 256 + 256 * 256 + 256 + 2 * 256 + 2


class Mlp(ctypes.Structure):
    _fields_ = [('params', _c_void_p), ('grads', _c_void_p), ('adam_m', _c_void_p),
                ('adam_v', _c_void_p), ('w1b', _c_void_p), ('w2b', _c_void_p),
                ('w2tb', _c_void_p)]

# name -> (restype, argtypes); mirrors include/rqsqd.h
_P = ctypes.POINTER
SIGNATURES = {
    'rq_subspace_sizes': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, _P(ctypes.c_int32)]),
    'rq_presence_bits': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, _P(ctypes.c_int32)]),
    'rq_scratch_size': (ctypes.c_int, [ctypes.c_int64, _P(ctypes.c_size_t)]),
    'rq_subspace_build': (ctypes.c_int, [_P(Subspace), _c_void_p, _c_void_p]),
    'rq_xsource': (ctypes.c_int, [_P(Subspace), _c_void_p, ctypes.c_int32, _c_void_p, _c_void_p]),
    'rq_diagonal': (ctypes.c_int, [_c_void_p, ctypes.c_int64, _c_void_p, _c_void_p,
                                   ctypes.c_int32, _c_void_p, _c_void_p]),
    'rq_pack_states': (ctypes.c_int, [_c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int64,
                                      _c_void_p, _c_void_p]),
    'rq_uniquify_scratch_size': (ctypes.c_int, [ctypes.c_int64, _P(ctypes.c_size_t)]),
    'rq_uniquify': (ctypes.c_int, [_c_void_p, ctypes.c_int64, _c_void_p, _P(ctypes.c_int64),
                                   _c_void_p, _c_void_p]),
    'rq_terms_upload': (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _c_void_p, _c_void_p,
                                       _c_void_p, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                                       _c_void_p, _c_void_p, _P(Terms), _c_void_p]),
    'rq_terms_hash': (ctypes.c_int, [_P(Terms), _c_void_p, _c_void_p]),
    'rq_line_filter_bits': (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, _P(ctypes.c_int32)]),
    'rq_terms_group_scratch_size': (ctypes.c_int, [ctypes.c_int64, _P(ctypes.c_size_t)]),
    'rq_terms_group': (ctypes.c_int, [ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p,
                                      ctypes.c_int32, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                                      _P(ctypes.c_int64), _P(ctypes.c_int64),
                                      _P(ctypes.c_int32), _c_void_p, _c_void_p]),
    'rq_conn_build': (ctypes.c_int, [_P(Operator), _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                                     ctypes.c_int32, _P(ctypes.c_int64), _c_void_p, _c_void_p]),
    'rq_matvec': (ctypes.c_int, [_P(Operator), ctypes.c_int32, _c_void_p, _c_void_p, _c_void_p,
                                 _c_void_p]),
    'rq_fullspace_matvec': (ctypes.c_int, [_P(Terms), ctypes.c_int32, ctypes.c_int32, _c_void_p,
                                           _c_void_p, _c_void_p]),
    'rq_lobpcg_workspace_size': (ctypes.c_int, [ctypes.c_int64, _P(LobpcgParams),
                                                _P(ctypes.c_size_t)]),
    'rq_lobpcg_solve': (ctypes.c_int, [_P(Operator), _P(LobpcgParams), _c_void_p, _c_void_p,
                                       _c_void_p, _P(LobpcgResult), _c_void_p]),
    'rq_lobpcg_solve_cb': (ctypes.c_int, [ctypes.c_int64, _c_void_p, _c_void_p, _P(LobpcgParams),
                                          _c_void_p, _c_void_p, _c_void_p, _P(LobpcgResult),
                                          _c_void_p]),
    'rq_lobpcg_solve_noalloc': (ctypes.c_int, [_P(Operator), _P(LobpcgParams), _c_void_p,
                                               _c_void_p, _P(LobpcgResult), _c_void_p]),
    'rq_eigenpair_3x3': (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p]),
    'rq_batch_build': (ctypes.c_int, [_P(Batch), _c_void_p, _c_void_p]),
    'rq_batch_conn_build': (ctypes.c_int, [_P(Batch), _c_void_p, _c_void_p, _c_void_p,
                                           _P(ctypes.c_int64), _c_void_p, _c_void_p]),
    'rq_batch_matvec': (ctypes.c_int, [_P(Batch), ctypes.c_int32, _c_void_p, _c_void_p, _c_void_p,
                                       _c_void_p]),
    'rq_batch_workspace_size': (ctypes.c_int, [_P(Batch), _P(LobpcgParams), _P(ctypes.c_size_t)]),
    'rq_batch_solve': (ctypes.c_int, [_P(Batch), _P(LobpcgParams), _c_void_p, _c_void_p, _c_void_p,
                                      _P(LobpcgResult), _c_void_p]),
    'rq_mlp_workspace_size': (ctypes.c_int, [ctypes.c_int64, _P(ctypes.c_size_t)]),
    'rq_mlp_sync': (ctypes.c_int, [_P(Mlp), _c_void_p]),
    'rq_mlp_features': (ctypes.c_int, [_c_void_p, ctypes.c_int64, ctypes.c_double, _c_void_p,
                                       _c_void_p]),
    'rq_mlp_sample': (ctypes.c_int, [_c_void_p, ctypes.c_int64, _c_void_p, _c_void_p,
                                     ctypes.c_int32, ctypes.c_uint64, ctypes.c_int64,
                                     ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    'rq_mlp_fwd': (ctypes.c_int, [_P(Mlp), ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p,
                                  _c_void_p]),
    'rq_mlp_infer': (ctypes.c_int, [_P(Mlp), ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p,
                                    _c_void_p]),
    'rq_mlp_loss': (ctypes.c_int, [ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p, _c_void_p,
                                   _c_void_p, _c_void_p]),
    'rq_mlp_bwd': (ctypes.c_int, [_P(Mlp), ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p,
                                  _c_void_p]),
    'rq_mlp_train': (ctypes.c_int, [_P(Mlp), ctypes.c_int64, _c_void_p, _c_void_p, _c_void_p,
                                    _c_void_p, _c_void_p, _c_void_p, _c_void_p]),
    'rq_mlp_step': (ctypes.c_int, [_P(Mlp), ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, _c_void_p]),
    'rq_mlp_warm_start': (ctypes.c_int, [ctypes.c_int64, _c_void_p, ctypes.c_int32, _c_void_p,
                                         _c_void_p]),
    'rq_bf16_gemm': (ctypes.c_int, [_c_void_p, ctypes.c_int64, _c_void_p, ctypes.c_int64,
                                    ctypes.c_int64, ctypes.c_int32, ctypes.c_int64, _c_void_p,
                                    _c_void_p, _c_void_p]),
    'rq_svsim': (ctypes.c_int, [_c_void_p, _c_void_p, _c_void_p, _c_void_p, ctypes.c_int32,
                                ctypes.c_int32, _c_void_p, _c_void_p, _c_void_p]),
    'rq_last_error': (ctypes.c_char_p, []),
    'rq_version': (ctypes.c_int, []),
}

MATVEC_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                             ctypes.c_void_p, ctypes.c_void_p)

_lock = threading.Lock()
_lib = None


class RqError(RuntimeError):
    """Nonzero status from the C ABI (code and rq_last_error message)."""

    def __init__(self, code, msg):
        super().__init__(f'[rq error {code}] {msg}')
        self.code = code


def lib():
    """Load librqsqd.so (built by ``rqutils_gb300._build.build()``); raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f'{LIB_PATH} is missing: build it with `python -m rqutils_gb300._build` '
                    '(there is no CPU fallback)')
            handle = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(rc, what=''):
    if rc != OK:
        msg = lib().rq_last_error().decode(errors='replace')
        raise RqError(rc, f'{what}: {msg}' if what else msg)
    return rc


def ptr(t):
    """Device address of a torch tensor as an int (None -> NULL)."""
    return None if t is None else int(t.data_ptr())


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)
