"""Tensor-core MLP of the learned warm start (rq_mlp_*, rq_bf16_gemm) against PyTorch FP32
references of the same operations (same BF16 roundings)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _gemm(A, B, K):
    import ctypes
    import torch
    from rqutils_gb300 import _lib as L
    M, N = A.shape[0], B.shape[0]
    C = torch.empty((M, N), dtype=torch.float32, device='cuda')
    ws = torch.zeros(64, dtype=torch.uint8, device='cuda')
    L.check(L.lib().rq_bf16_gemm(L.ptr(A), A.stride(0), L.ptr(B), B.stride(0), M, N, K, L.ptr(C),
                                 L.ptr(ws), L.stream_ptr()), 'rq_bf16_gemm')
    torch.cuda.synchronize()
    assert int(ws[:4].view(torch.int32).item()) == 0
    return C


@pytest.mark.parametrize('N', [64, 256])
@pytest.mark.parametrize('M,K,lda', [(128, 64, 64), (300, 192, 192), (257, 128, 256), (500, 512, 520),
                                     (64, 320, 320)])
def test_bf16_gemm_exact_on_small_integers(N, M, K, lda):
    """Integer operands in [-3, 3]: every product and partial sum is exact in FP32, so the
    tensor-core result must equal the FP32 product bit for bit (layouts, descriptors, K loop,
    ragged row tile; B kept in shared memory for K <= 256, streamed with A beyond, a 64-row A)."""
    import torch
    g = torch.Generator().manual_seed(M + N + K)
    Afull = torch.randint(-3, 4, (M, lda), generator=g).to(torch.bfloat16).cuda()
    B = torch.randint(-3, 4, (N, K), generator=g).to(torch.bfloat16).cuda()
    C = _gemm(Afull, B, K)
    ref = Afull[:, :K].float() @ B.float().T
    assert torch.equal(C, ref)


def test_bf16_gemm_random_values():
    import torch
    g = torch.Generator().manual_seed(7)
    A = torch.randn((1000, 512), generator=g).to(torch.bfloat16).cuda()
    B = torch.randn((256, 512), generator=g).to(torch.bfloat16).cuda()
    C = _gemm(A, B, 512)
    ref = A.double() @ B.double().T
    err = (C.double() - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


def _reference_forward(m, x):
    import torch
    import torch.nn.functional as F
    W1, b1, W2, b2, W3, b3 = m.views()
    z1 = x.float() @ m.w1b.float().T + b1
    h1b = F.gelu(z1, approximate='tanh').to(torch.bfloat16).float()
    z2 = h1b @ m.w2b.float().T + b2
    out = F.gelu(z2, approximate='tanh') @ W3.T + b3
    return out, z1, h1b, z2


def _features(rows, seed):
    import torch
    from rqutils_gb300.warmstart import features_reference
    rng = np.random.default_rng(seed)
    s = rng.integers(0, 1 << 32, size=rows, dtype=np.uint64)
    U = rng.uniform(2, 8, size=rows)
    f = np.stack([features_reference(s[i:i + 1], U[i])[0] for i in range(rows)])
    return torch.as_tensor(f).to(torch.bfloat16).cuda()


def test_features_match_host_restatement():
    import torch
    from rqutils_gb300.warmstart import WarmStartMLP, features_reference
    from rqutils_gb300 import _lib as L
    rng = np.random.default_rng(2)
    s = np.sort(rng.choice(1 << 32, size=1000, replace=False).astype(np.uint64))
    x = torch.empty((1000, 64), dtype=torch.bfloat16, device='cuda')
    st = torch.as_tensor(s.view(np.int64)).cuda()
    L.check(L.lib().rq_mlp_features(L.ptr(st), 1000, 3.7, L.ptr(x), L.stream_ptr()), 'features')
    ref = torch.as_tensor(features_reference(s, 3.7)).to(torch.bfloat16)
    assert torch.equal(x.cpu(), ref)


@pytest.mark.parametrize('rows', [128, 1000, 4096])
def test_forward_matches_torch(rows):
    import torch
    from rqutils_gb300.warmstart import WarmStartMLP
    m = WarmStartMLP(seed=3)
    x = _features(rows, rows)
    out = m.forward(x)
    ref = _reference_forward(m, x)[0]
    m.check_errors()
    err = (out - ref).abs().max().item()
    assert err < 2e-3 * max(1., ref.abs().max().item()), err
    # inference without the stored activations gives the same outputs bit for bit
    assert torch.equal(m.infer(x), out)


def test_backward_matches_torch():
    """Weight gradients of a random output gradient against the same chain rule in PyTorch
    (BF16 operands where the kernels use them, FP32 accumulation)."""
    import torch
    import torch.nn.functional as F
    from rqutils_gb300.warmstart import (OFF_B1, OFF_B2, OFF_B3, OFF_W1, OFF_W2, OFF_W3,
                                         NPARAMS, WarmStartMLP)
    rows = 2048
    m = WarmStartMLP(seed=4)
    x = _features(rows, 11)
    out = m.forward(x)
    g = torch.Generator().manual_seed(5)
    dout = (torch.randn((rows, 2), generator=g) / rows).cuda()
    m.backward(x.T.contiguous(), dout)
    torch.cuda.synchronize()
    m.check_errors()
    W1, b1, W2, b2, W3, b3 = m.views()
    _, z1, h1b, z2 = _reference_forward(m, x)

    def dgelu(z):  # derivative of the tanh form of GELU
        k0, k1 = math.sqrt(2 / math.pi), 0.044715
        t = torch.tanh(k0 * (z + k1 * z ** 3))
        return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * k0 * (1 + 3 * k1 * z * z)

    z2b = z2.to(torch.bfloat16).float()
    dz2 = (dout @ W3) * dgelu(z2b)
    dz2b = dz2.to(torch.bfloat16).float()
    ref = torch.zeros(NPARAMS, dtype=torch.float32, device='cuda')
    ref[OFF_W3:OFF_B3] = (dout.T @ F.gelu(z2b, approximate='tanh')).reshape(-1)
    ref[OFF_B3:] = dout.sum(0)
    ref[OFF_B2:OFF_W3] = dz2.sum(0)
    ref[OFF_W2:OFF_B2] = (dz2b.T @ h1b).reshape(-1)
    dz1 = (dz2b @ m.w2b.float()) * dgelu(z1.to(torch.bfloat16).float())
    ref[OFF_B1:OFF_W2] = dz1.sum(0)
    ref[OFF_W1:OFF_B1] = (dz1.to(torch.bfloat16).float().T @ x.float()).reshape(-1)
    for a, b, name in [(OFF_W1, OFF_B1, 'W1'), (OFF_B1, OFF_W2, 'b1'), (OFF_W2, OFF_B2, 'W2'),
                       (OFF_B2, OFF_W3, 'b2'), (OFF_W3, OFF_B3, 'W3'), (OFF_B3, NPARAMS, 'b3')]:
        e = (m.grads[a:b] - ref[a:b]).norm().item() / max(ref[a:b].norm().item(), 1e-30)
        assert e < 2e-2, (name, e)


@pytest.mark.parametrize('rows', [128, 4096, 20480])
def test_fused_train_step_matches_separate_calls(rows):
    """rq_mlp_train (loss and head backward in layer 2's epilogue, split-K weight gradients)
    against rq_mlp_fwd + rq_mlp_loss + rq_mlp_bwd on the same minibatch: the same loss and
    outputs, and gradients equal up to the BF16 rounding of Z2 that only the separate path does."""
    import torch
    from rqutils_gb300.warmstart import (OFF_B1, OFF_B2, OFF_B3, OFF_W1, OFF_W2, OFF_W3,
                                         NPARAMS, WarmStartMLP)
    m = WarmStartMLP(seed=14)
    x = _features(rows, 21) if rows <= 4096 else _features(4096, 21).repeat(rows // 4096, 1)
    g = torch.Generator().manual_seed(22)
    tgt = torch.stack([torch.randn(rows, generator=g) - 2.,
                       torch.where(torch.rand(rows, generator=g) < 0.5, -1., 1.),
                       torch.rand(rows, generator=g) * 2. + 0.05], 1).cuda()
    xt = x.T.contiguous()
    out = m.forward(x)
    loss_a = torch.zeros(1, dtype=torch.float64, device='cuda')
    dout = m.loss(out, tgt, loss=loss_a)
    m.backward(xt, dout)
    ga = m.grads.clone()
    out_b = torch.empty_like(out)
    loss_b = torch.zeros(1, dtype=torch.float64, device='cuda')
    m.train_step(x, xt, tgt, out=out_b, loss=loss_b)
    torch.cuda.synchronize()
    m.check_errors()
    assert torch.allclose(out_b, out, rtol=0, atol=1e-5)
    o, t = out.double(), tgt.double()
    z = -t[:, 1] * o[:, 1]
    loss_ref = (t[:, 2] * ((o[:, 0] - t[:, 0]) ** 2 + torch.nn.functional.softplus(z))).mean()
    assert abs(loss_a.item() - loss_ref.item()) <= 1e-5 * abs(loss_ref.item())
    assert abs(loss_b.item() - loss_a.item()) <= 1e-6 * abs(loss_a.item())
    gb = m.grads
    for a, b, name in [(OFF_W1, OFF_B1, 'W1'), (OFF_B1, OFF_W2, 'b1'), (OFF_W2, OFF_B2, 'W2'),
                       (OFF_B2, OFF_W3, 'b2'), (OFF_W3, OFF_B3, 'W3'), (OFF_B3, NPARAMS, 'b3')]:
        e = (gb[a:b] - ga[a:b]).norm().item() / max(ga[a:b].norm().item(), 1e-30)
        assert e < 1e-2, (name, e)
    # the weight gradients are deterministic: a second call gives the same bits
    g1 = gb.clone()
    m.train_step(x, xt, tgt)
    torch.cuda.synchronize()
    assert torch.equal(m.grads, g1)


def test_adam_step_and_bf16_copies():
    import torch
    from rqutils_gb300.warmstart import NPARAMS, WarmStartMLP
    m = WarmStartMLP(seed=6)
    p0 = m.params.clone()
    g = torch.randn(NPARAMS, generator=torch.Generator().manual_seed(1)).cuda()
    m.grads.copy_(g)
    m.step(1e-2)
    mm = 0.1 * g
    vv = 0.001 * g * g
    ref = p0 - 1e-2 * (mm / 0.1) / (torch.sqrt(vv / 0.001) + 1e-8)
    torch.cuda.synchronize()
    assert torch.allclose(m.params, ref, rtol=1e-5, atol=1e-6)
    W1, b1, W2, b2, W3, b3 = m.views()
    assert torch.equal(m.w1b, W1.to(torch.bfloat16))
    assert torch.equal(m.w2b, W2.to(torch.bfloat16))
    assert torch.equal(m.w2tb, W2.T.contiguous().to(torch.bfloat16))


def test_training_fits_a_smooth_family():
    """Synthetic family psi_U(s) ~ sign(s) exp(-U w(s) / 8): the loss falls and the warm start
    of a held-out U overlaps its target."""
    import torch
    from rqutils_gb300.warmstart import WarmStartMLP
    rng = np.random.default_rng(8)
    D = 4096
    S = np.sort(rng.choice(1 << 20, size=D, replace=False).astype(np.uint64))
    w = np.bitwise_count(S & np.uint64(0x3FF)).astype(np.float64)
    sign = np.where(np.bitwise_count(S & np.uint64(0xF)) % 2 == 0, 1., -1.)

    def psi_of(U):
        v = sign * np.exp(-U * w / 8.)
        return v / np.linalg.norm(v)

    Us = np.linspace(2, 8, 16)
    psi = torch.as_tensor(np.stack([psi_of(u) for u in Us]), dtype=torch.float32)
    m = WarmStartMLP(seed=9)
    losses = m.fit(S, Us, psi, steps=300, batch=8192, lr=3e-3, log_every=50)
    assert losses[-1][1] < 0.5 * losses[0][1], losses
    x0 = m.warm_start(S, 5.1).cpu().numpy()
    t = psi_of(5.1)
    assert abs(np.dot(x0, t)) / np.linalg.norm(x0) > 0.9


def test_hubbard_family_and_learned_start_small():
    """Hubbard 4x2 family on a low-double-occupancy subspace: continuation ground states match
    dense diagonalisation; a network trained on 24 values of U starts held-out solves close to
    their ground states, in fewer LOBPCG iterations than random starts need, and they converge
    to the same energies."""
    import torch
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import hproj
    from rqutils_gb300.warmstart import WarmStartMLP, evaluate_starts, hubbard_family
    from rqutils_gb300.workloads import hubbard_jw, low_double_occupancy_states
    rng = np.random.default_rng(12)
    S = low_double_occupancy_states(rng, 1000, Ns=8)
    Us = np.linspace(2., 8., 24)
    psi, eig, its = hubbard_family(S, Us, Lx=4, Ly=2)
    for k in (0, 11, 23):
        h = PauliSumXZ.from_paulisum(hubbard_jw(4, 2, 1.0, Us[k]), force_real=True, add_padding=True)
        e_dense = np.linalg.eigvalsh(hproj(h, S).toarray())[0]
        assert abs(eig[k] - e_dense) <= 1e-6 * abs(e_dense), (k, eig[k], e_dense)
    m = WarmStartMLP(seed=1)
    m.fit(S, Us, psi, steps=400, batch=4096, lr=3e-3)
    res = evaluate_starts(m, S, [3.3, 4.7, 6.1], Lx=4, Ly=2)
    for rl, rr in zip(res['learned'], res['random']):
        assert rl['converged'] and rr['converged']
        assert rl['start_overlap'] > 0.8, rl
        assert abs(rl['eigval'] - rr['eigval']) <= 1e-9 * abs(rr['eigval'])
        assert rl['rel_residual'] < 1e-7
        # what the trained network gains: fewer iterations than from a random start
        assert rl['iterations'] < rr['iterations'], (rl, rr)
    assert (sum(r['iterations'] for r in res['learned']) <=
            0.8 * sum(r['iterations'] for r in res['random'])), res
