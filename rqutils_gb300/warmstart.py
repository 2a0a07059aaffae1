r"""Learned LOBPCG start vectors (``rq_mlp_*``).

The reference starts LOBPCG from a one-hot vector at the lowest diagonal entry
(``rqutils/sqd.py:373-398``).  For a family of problems that share a subspace and differ in one
Hamiltonian parameter U (Hubbard models at several interaction strengths), a small network can
predict the ground state of a new U from ground states already solved:

    f(bits(s), U) = (log(sqrt(D) |psi(s)|), sign logit)       x0(s) = sign * exp(log-amplitude)

``WarmStartMLP`` holds the network (64 -> 256 -> 256 -> 2, GELU; BF16 weights on the tcgen05
tensor cores, FP32 master weights and Adam state) and trains it on (state, U) pairs sampled from
solved ground states; every step (sampling, forward, loss, backward, Adam) is a call into
librqsqd.so on the device.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib as L
from .device import TORCH_DTYPE, VTYPE_OF, _u64_tensor, default_device

OFF_W1 = 0
OFF_B1 = OFF_W1 + 256 * 64
OFF_W2 = OFF_B1 + 256
OFF_B2 = OFF_W2 + 256 * 256
OFF_W3 = OFF_B2 + 256
OFF_B3 = OFF_W3 + 2 * 256
NPARAMS = OFF_B3 + 2
assert NPARAMS == L.MLP_NPARAMS


def init_params(seed=0):
    """He-style initial weights (N(0, 1 / fan_in)), zero biases, small output layer (FP32)."""
    g = torch.Generator().manual_seed(seed)
    p = torch.zeros(NPARAMS, dtype=torch.float32)
    p[OFF_W1:OFF_B1] = torch.randn(256 * 64, generator=g) / math.sqrt(36.)
    p[OFF_W2:OFF_B2] = torch.randn(256 * 256, generator=g) / math.sqrt(256.)
    p[OFF_W3:OFF_B3] = torch.randn(2 * 256, generator=g) * (0.1 / math.sqrt(256.))
    return p


class WarmStartMLP:
    def __init__(self, device=None, seed=0, params=None):
        self.device = device or default_device()
        dev = self.device
        p = init_params(seed) if params is None else torch.as_tensor(params, dtype=torch.float32)
        self.params = p.to(dev).contiguous()
        self.grads = torch.zeros(NPARAMS, dtype=torch.float32, device=dev)
        self.adam_m = torch.zeros(NPARAMS, dtype=torch.float32, device=dev)
        self.adam_v = torch.zeros(NPARAMS, dtype=torch.float32, device=dev)
        self.w1b = torch.empty((256, 64), dtype=torch.bfloat16, device=dev)
        self.w2b = torch.empty((256, 256), dtype=torch.bfloat16, device=dev)
        self.w2tb = torch.empty((256, 256), dtype=torch.bfloat16, device=dev)
        self.c = L.Mlp(params=L.ptr(self.params), grads=L.ptr(self.grads),
                       adam_m=L.ptr(self.adam_m), adam_v=L.ptr(self.adam_v),
                       w1b=L.ptr(self.w1b), w2b=L.ptr(self.w2b), w2tb=L.ptr(self.w2tb))
        L.check(L.lib().rq_mlp_sync(ctypes.byref(self.c), L.stream_ptr()), 'rq_mlp_sync')
        self.t = 0
        self._ws = None

    # ------------------------------------------------------------------------------------------
    def views(self):
        """FP32 parameter views: W1 (256, 64), b1, W2 (256, 256), b2, W3 (2, 256), b3."""
        p = self.params
        return (p[OFF_W1:OFF_B1].view(256, 64), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].view(256, 256),
                p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].view(2, 256), p[OFF_B3:])

    def workspace(self, rows):
        n = ctypes.c_size_t()
        L.check(L.lib().rq_mlp_workspace_size(int(rows), ctypes.byref(n)), 'rq_mlp_workspace_size')
        if self._ws is None or self._ws.numel() < n.value:
            self._ws = torch.empty(int(n.value), dtype=torch.uint8, device=self.device)
        return self._ws

    def forward(self, x, out=None, stream=None):
        """out (rows, 2) FP32 for BF16 features x (rows, 64); keeps activations for backward."""
        rows = x.shape[0]
        ws = self.workspace(rows)
        if out is None:
            out = torch.empty((rows, 2), dtype=torch.float32, device=self.device)
        L.check(L.lib().rq_mlp_fwd(ctypes.byref(self.c), rows, L.ptr(x), L.ptr(out), L.ptr(ws),
                                   L.stream_ptr(stream)), 'rq_mlp_fwd')
        return out

    def infer(self, x, out=None, stream=None):
        """out (rows, 2) FP32 for BF16 features x (rows, 64), keeping no activations."""
        rows = x.shape[0]
        ws = self.workspace(rows)
        if out is None:
            out = torch.empty((rows, 2), dtype=torch.float32, device=self.device)
        L.check(L.lib().rq_mlp_infer(ctypes.byref(self.c), rows, L.ptr(x), L.ptr(out), L.ptr(ws),
                                     L.stream_ptr(stream)), 'rq_mlp_infer')
        return out

    def loss(self, out, tgt, dout=None, loss=None, stream=None):
        rows = out.shape[0]
        ws = self.workspace(rows)
        if dout is None:
            dout = torch.empty_like(out)
        L.check(L.lib().rq_mlp_loss(rows, L.ptr(out), L.ptr(tgt), L.ptr(dout), L.ptr(loss),
                                    L.ptr(ws), L.stream_ptr(stream)), 'rq_mlp_loss')
        return dout

    def backward(self, xt, dout, stream=None):
        """grads from dout (rows, 2) and the features transposed xt (64, rows)."""
        rows = dout.shape[0]
        ws = self.workspace(rows)
        L.check(L.lib().rq_mlp_bwd(ctypes.byref(self.c), rows, L.ptr(xt), L.ptr(dout), L.ptr(ws),
                                   L.stream_ptr(stream)), 'rq_mlp_bwd')
        return self.grads

    def train_step(self, x, xt, tgt, out=None, loss=None, stream=None):
        """Forward, loss and backward of one minibatch in one call (rq_mlp_train): grads from
        features x (rows, 64), their transpose xt (64, rows) and targets tgt (rows, 3).  The
        loss (device double, shape (1,)) is written when ``loss`` is given."""
        rows = x.shape[0]
        ws = self.workspace(rows)
        L.check(L.lib().rq_mlp_train(ctypes.byref(self.c), rows, L.ptr(x), L.ptr(xt), L.ptr(tgt),
                                     L.ptr(out), L.ptr(loss), L.ptr(ws), L.stream_ptr(stream)),
                'rq_mlp_train')
        return self.grads

    def step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        self.t += 1
        L.check(L.lib().rq_mlp_step(ctypes.byref(self.c), self.t, float(lr), float(beta1),
                                    float(beta2), float(eps), L.stream_ptr(stream)), 'rq_mlp_step')

    def check_errors(self):
        if self._ws is not None:
            flag = int(self._ws[:4].view(torch.int32).item())
            if flag:
                raise L.RqError(flag, 'an MLP kernel reported an error')

    # ------------------------------------------------------------------------------------------
    def fit(self, states, U, psi, steps=2000, batch=65536, lr=2e-3, lr_min=1e-4, seed=1,
            log_every=0):
        """Train on ground states psi (P, D) FP32 of the problems with parameters U (P,) over
        the sorted states (D,).  Cosine learning-rate decay.  Returns the logged losses."""
        dev = self.device
        batch = int(batch + 127) // 128 * 128
        S = states if isinstance(states, torch.Tensor) else _u64_tensor(states, dev)
        Ut = torch.as_tensor(np.asarray(U, dtype=np.float64), device=dev)
        psi = psi.to(dev, torch.float32).contiguous()
        P, D = psi.shape
        x = torch.empty((batch, 64), dtype=torch.bfloat16, device=dev)
        xt = torch.empty((64, batch), dtype=torch.bfloat16, device=dev)
        tgt = torch.empty((batch, 3), dtype=torch.float32, device=dev)
        lossv = torch.zeros(1, dtype=torch.float64, device=dev)
        lib = L.lib()
        st = L.stream_ptr()
        logged = []
        for k in range(steps):
            L.check(lib.rq_mlp_sample(L.ptr(S), D, L.ptr(Ut), L.ptr(psi), P, seed, k, batch,
                                      L.ptr(x), L.ptr(xt), L.ptr(tgt), st), 'rq_mlp_sample')
            want = log_every and (k % log_every == 0 or k == steps - 1)
            self.train_step(x, xt, tgt, loss=lossv if want else None)
            frac = k / max(1, steps - 1)
            self.step(lr_min + 0.5 * (lr - lr_min) * (1. + math.cos(math.pi * frac)))
            if want:
                logged.append((k, float(lossv.item())))
        self.check_errors()
        return logged

    def predict(self, states, U, out=None):
        """Network outputs (D, 2) on every state for one U."""
        dev = self.device
        S = states if isinstance(states, torch.Tensor) else _u64_tensor(states, dev)
        D = S.numel()
        x = torch.empty((D, 64), dtype=torch.bfloat16, device=dev)
        L.check(L.lib().rq_mlp_features(L.ptr(S), D, float(U), L.ptr(x), L.stream_ptr()),
                'rq_mlp_features')
        return self.infer(x, out)

    def warm_start(self, states, U, dtype=torch.float64):
        """Start vector sign * exp(log-amplitude) on every state for one U."""
        out = self.predict(states, U)
        D = out.shape[0]
        x0 = torch.empty(D, dtype=dtype, device=self.device)
        L.check(L.lib().rq_mlp_warm_start(D, L.ptr(out), VTYPE_OF[dtype], L.ptr(x0),
                                          L.stream_ptr()), 'rq_mlp_warm_start')
        return x0


def features_reference(states, U):
    """Host copy of the network input (rows, 64) FP32 (the oracle of rq_mlp_features)."""
    s = np.asarray(states, dtype=np.uint64)
    f = np.zeros((len(s), 64), dtype=np.float32)
    bits = ((s[:, None] >> np.arange(32, dtype=np.uint64)) & np.uint64(1)).astype(np.float32)
    f[:, :32] = 2. * bits - 1.
    u = (np.asarray(U, dtype=np.float64) - 5.) / 3.
    u = np.broadcast_to(u, (len(s),))
    f[:, 32], f[:, 33], f[:, 34] = u, u * u, u * u * u
    return f


# ---------------------------------------------------------------------------------------------
# Hubbard family: training data and evaluation of start vectors
# ---------------------------------------------------------------------------------------------
def _hubbard_operator(sub, U, Lx, Ly, t, periodic, device):
    from .device import DeviceOperator, DeviceTerms
    from .paulis.symplectic import PauliSumXZ
    from .workloads import hubbard_jw
    ham = PauliSumXZ.from_paulisum(hubbard_jw(Lx, Ly, t, float(U), periodic), force_real=True,
                                   add_padding=True)
    return DeviceOperator(DeviceTerms(ham, device=device), sub, mode='conn')


def hubbard_family(S, Us, Lx=4, Ly=4, t=1.0, periodic=True, target_rel=1e-7, maxiter=5000,
                   seed=0, device=None):
    """Ground states of the Hubbard models at every U on the sorted subspace S, solved by the
    plain LOBPCG solver with continuation: U ascending, each solve started from the previous
    ground state (the first from a seeded random vector).  Signs are aligned with the previous
    state (the first has its largest component positive).  Returns (psi (P, D) FP32 in the
    order of Us, eigenvalues, iterations)."""
    from .device import DeviceSubspace
    from .ground_locg import lobpcg_solve
    dev = device or default_device()
    sub = DeviceSubspace(S, num_qubits=2 * Lx * Ly, device=dev)
    Us = np.asarray(Us, dtype=np.float64)
    psi = torch.empty((len(Us), sub.D), dtype=torch.float32, device=dev)
    eig = np.zeros(len(Us))
    its = np.zeros(len(Us), dtype=np.int64)
    x = torch.as_tensor(np.random.default_rng(seed).normal(size=sub.D), device=dev)
    prev = None
    for i in np.argsort(Us, kind='stable'):
        op = _hubbard_operator(sub, Us[i], Lx, Ly, t, periodic, dev)
        e, x, info = lobpcg_solve(op, x, maxiter=maxiter, target_rel=target_rel, variant='fast')
        if prev is None:
            if x[int(torch.argmax(x.abs()))] < 0:
                x = -x
        elif torch.dot(x, prev) < 0:
            x = -x
        prev = x
        psi[i] = x.float()
        eig[i] = e
        its[i] = info['niter']
    return psi, eig, its


def evaluate_starts(model, S, Us, Lx=4, Ly=4, t=1.0, periodic=True, target_rel=1e-8,
                    maxiter=5000, seed=0, device=None, mixed=True, variant='fast', jacobi=False):
    """LOBPCG to |r| <= target_rel |theta| on each U from three start vectors: the network's
    ('learned', inference included in the time), a seeded random vector ('random') and the
    reference's one-hot at the lowest diagonal entry ('reference').  Returns {start: [dict]}."""
    import time
    from .device import DeviceSubspace
    from .ground_locg import lobpcg_solve
    dev = device or default_device()
    sub = DeviceSubspace(S, num_qubits=2 * Lx * Ly, device=dev)
    rng = np.random.default_rng(seed)
    res = {'learned': [], 'random': [], 'reference': []}
    for U in np.asarray(Us, dtype=np.float64):
        op = _hubbard_operator(sub, U, Lx, Ly, t, periodic, dev)
        xr = torch.as_tensor(rng.normal(size=sub.D), device=dev)
        for name in res:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if name == 'learned':
                x0 = model.warm_start(sub.states, U, torch.float64)
            elif name == 'random':
                x0 = xr
            else:
                x0 = torch.zeros(sub.D, dtype=torch.float64, device=dev)
                x0[int(torch.argmin(op.diag0))] = 1.
            e, x, info = lobpcg_solve(op, x0, maxiter=maxiter, target_rel=target_rel,
                                      variant=variant, mixed=mixed, jacobi=jacobi)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            ax = op.matvec(x)
            rel = float(torch.linalg.vector_norm(ax - e * x) / abs(e))
            ov = None
            if name == 'learned':
                ov = float(abs(torch.dot(x0, x)) / torch.linalg.vector_norm(x0))
            res[name].append({'U': float(U), 'iterations': info['niter'], 'time_s': dt,
                              'eigval': e, 'rel_residual': rel, 'converged': info['converged'],
                              'start_overlap': ov})
    return res
