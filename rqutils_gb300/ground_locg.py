r"""Single-vector LOBPCG on the GPU -- drop-in for ``rqutils.ground_locg``.

``ground_locg(mat, xinit, args=(), maxiter=1000, tol=None, vspace=None, log_level=WARNING)``
keeps the reference signature and return value ``(eigval, eigvec, niter)``
(``rqutils/ground_locg.py:128-157``).  The iteration -- projection (380-421), Rayleigh-Ritz with
the analytic 2x2 / 3x3 eigenpairs (235-255, 424-471), update and convergence test (288-341) -- runs
as fused CUDA kernels with FP64 reductions and device-resident scalars (``rq_lobpcg_solve``):

* ``mat`` a ``DeviceOperator``: the matvec is the library's own kernel and chunks of iterations
  are replayed as CUDA graphs;
* ``mat`` a callable ``f(x, *args)`` on torch CUDA tensors, or a dense matrix: the matvec is
  called back from the solver (``rq_lobpcg_solve_cb``).

Extra keyword arguments (not in the reference): ``variant`` ('reference': four matvecs per
iteration as the reference; 'fast': one, with A x and A y carried by linearity), ``precision``
('fp64' or 'mixed': a 32-bit phase, then FP64 refinement), ``target_rel`` (also stop when
|r| <= target_rel |theta|), ``jacobi`` (diagonal preconditioner), ``use_graph``, ``restart``
('fast' with a DeviceOperator: restart the step from x every that many iterations of a phase).
"""
import ctypes
import logging

import numpy as np
import torch

from . import _lib as L
from .device import DeviceOperator, TORCH_DTYPE, VTYPE_OF, default_device

LOG = logging.getLogger(__name__)

_VARIANTS = {'reference': L.LOBPCG_REFERENCE, 'fast': L.LOBPCG_FAST}


def _params(D, vtype, maxiter, tol, tol_dim, variant, mixed, target_rel, switch_rel, refresh,
            use_graph, jacobi, guard=True, restart=0):
    return L.LobpcgParams(maxiter=int(maxiter), variant=_VARIANTS[variant], vtype=vtype,
                          mixed=int(bool(mixed)), tol=float(tol or 0.),
                          tol_dim=float(tol_dim or 0.), switch_rel=float(switch_rel),
                          target_rel=float(target_rel or 0.), refresh=int(refresh),
                          use_graph=int(use_graph) if use_graph in (0, 1, 2) else 1,
                          jacobi=int(bool(jacobi)),
                          guard=int(bool(guard)), restart=int(restart or 0))


def _workspace(owner, D, prm, device):
    n = ctypes.c_size_t()
    L.check(L.lib().rq_lobpcg_workspace_size(int(D), ctypes.byref(prm), ctypes.byref(n)),
            'rq_lobpcg_workspace_size')
    ws = getattr(owner, '_lobpcg_ws', None) if owner is not None else None
    if ws is None or ws.numel() < n.value or ws.device != device:
        ws = torch.empty(int(n.value), dtype=torch.uint8, device=device)
        if owner is not None:
            owner._lobpcg_ws = ws
    return ws


def _info(res):
    return dict(eigval=res.eigval, resnorm=res.resnorm, axnorm=res.axnorm, niter=res.niter,
                niter_lo=res.niter_lo, converged=bool(res.converged), status=res.status)


def lobpcg_solve(op: DeviceOperator, x0, maxiter=1000, tol=None, tol_dim=None,
                 variant='reference', mixed=False, target_rel=None, switch_rel=1e-5, refresh=32,
                 use_graph=True, jacobi=False, guard=True, stream=None, restart=0):
    """Run rq_lobpcg_solve on a DeviceOperator from the device vector x0 (its dtype selects the
    value type).  ``restart`` (FAST variant): restart the step from x every that many iterations
    of a phase (0 = never, as the reference).  Returns (eigval, x, info)."""
    x0 = x0.contiguous()
    vt = VTYPE_OF[x0.dtype]
    prm = _params(op.D, vt, maxiter, tol, tol_dim, variant, mixed, target_rel, switch_rel,
                  refresh, use_graph, jacobi, guard, restart)
    ws = _workspace(op, op.D, prm, op.device)
    xout = torch.empty_like(x0)
    res = L.LobpcgResult()
    L.check(L.lib().rq_lobpcg_solve(ctypes.byref(op.c), ctypes.byref(prm), L.ptr(ws), L.ptr(x0),
                                    L.ptr(xout), ctypes.byref(res), L.stream_ptr(stream)),
            'rq_lobpcg_solve')
    op.check_errors()
    return res.eigval, xout, _info(res)


def lobpcg_solve_callable(matvec, x0, maxiter=1000, tol=None, tol_dim=None, mixed=False,
                          target_rel=None, switch_rel=1e-5, stream=None):
    """rq_lobpcg_solve_cb with a Python matvec on torch CUDA tensors."""
    x0 = x0.contiguous()
    D = x0.numel()
    vt = VTYPE_OF[x0.dtype]
    prm = _params(D, vt, maxiter, tol, tol_dim, 'reference', mixed, target_rel, switch_rel, 32,
                  False, False)
    ws = _workspace(None, D, prm, x0.device)
    base = ws.data_ptr()
    errors = []

    def cb(_ctx, vtype, xp, yp, sp):
        try:
            dt = TORCH_DTYPE[vtype]
            esz = torch.empty((), dtype=dt).element_size()
            xv = ws[xp - base: xp - base + D * esz].view(dt)
            yv = ws[yp - base: yp - base + D * esz].view(dt)
            stream = torch.cuda.ExternalStream(sp) if sp else torch.cuda.default_stream()
            with torch.cuda.stream(stream):
                yv.copy_(matvec(xv))
            return 0
        except Exception as exc:  # reported after the C call returns
            errors.append(exc)
            return 1

    fn = L.MATVEC_FN(cb)
    xout = torch.empty_like(x0)
    res = L.LobpcgResult()
    rc = L.lib().rq_lobpcg_solve_cb(D, fn, None, ctypes.byref(prm), L.ptr(ws), L.ptr(x0),
                                    L.ptr(xout), ctypes.byref(res), L.stream_ptr(stream))
    if errors:
        raise errors[0]
    L.check(rc, 'rq_lobpcg_solve_cb')
    return res.eigval, xout, _info(res)


def _is_int_scalar(v):
    if isinstance(v, (int, np.integer)):
        return True
    if isinstance(v, torch.Tensor):
        return v.ndim == 0 and not (v.is_floating_point() or v.is_complex())
    if isinstance(v, np.ndarray):
        return v.ndim == 0 and np.issubdtype(v.dtype, np.integer)
    return False


def ground_locg(mat, xinit, args=(), maxiter=1000, tol=None, vspace=None,
                log_level=logging.WARNING, *, variant='reference', precision=None,
                target_rel=None, jacobi=False, use_graph=True, tol_dim=None, restart=0,
                return_info=False):
    """Single-vector LOBPCG (ground_locg.py:128-157): lowest eigenvalue, eigenvector, iterations.

    ``xinit`` may be an integer (one-hot; with a callable ``mat`` it needs ``vspace=(dim, dtype)``,
    ground_locg.py:201-206).  NumPy inputs give NumPy outputs; torch inputs stay on the device.
    """
    as_numpy = not isinstance(xinit, torch.Tensor) and not (
        isinstance(mat, torch.Tensor))
    if isinstance(mat, DeviceOperator):
        device = mat.device
        dim = mat.D
        default_dtype = torch.float64 if mat.is_real else torch.complex128
    elif callable(mat):
        device = default_device()
        dim = vspace[0] if vspace is not None else None
        default_dtype = torch.complex128
    else:
        device = default_device()
        m = torch.as_tensor(mat).to(device)
        dim = m.shape[1]
        default_dtype = m.dtype
    if _is_int_scalar(xinit):
        if callable(mat) and not isinstance(mat, DeviceOperator):
            if vspace is None:
                raise ValueError('vspace is required when mat is callable and xinit is an integer')
            dtype = torch.as_tensor(np.zeros(0, dtype=vspace[1])).dtype
        else:
            dtype = default_dtype
        x0 = torch.zeros(dim, dtype=dtype, device=device)
        x0[int(xinit)] = 1
    else:
        x0 = torch.as_tensor(np.asarray(xinit) if as_numpy else xinit).to(device)
    mixed = precision == 'mixed'
    if isinstance(mat, DeviceOperator):
        eig, x, info = lobpcg_solve(mat, x0, maxiter=maxiter, tol=tol, tol_dim=tol_dim,
                                    variant=variant, mixed=mixed, target_rel=target_rel,
                                    jacobi=jacobi, use_graph=use_graph, restart=restart)
    else:
        if callable(mat):
            def mv(v):
                return mat(v, *args)
        else:
            cache = {}

            def mv(v):
                if v.dtype not in cache:
                    cache[v.dtype] = m.to(v.dtype)
                return cache[v.dtype] @ v
        eig, x, info = lobpcg_solve_callable(mv, x0, maxiter=maxiter, tol=tol, tol_dim=tol_dim,
                                             mixed=mixed, target_rel=target_rel)
    if log_level <= logging.DEBUG:
        LOG.debug('LOBPCG: %d iterations, residual %g', info['niter'], info['resnorm'])
    out = (float(eig), x.cpu().numpy() if as_numpy else x, int(info['niter']))
    return out + (info,) if return_info else out
