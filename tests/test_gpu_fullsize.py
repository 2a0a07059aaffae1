"""Size-independent properties at the benchmark sizes (GPU): the oracle cannot run these sizes,
so the checks are exact identities of the operator and of the front end."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _hermitian_checks(op, D, dtype, rng, tol):
    import torch
    x = torch.as_tensor(rng.normal(size=D) + 1j * rng.normal(size=D)).to(dtype).cuda()
    y = torch.as_tensor(rng.normal(size=D) + 1j * rng.normal(size=D)).to(dtype).cuda()
    hx, hy = op.matvec(x), op.matvec(y)
    a, b = 0.3 - 0.7j, -1.1 + 0.2j
    lin = op.matvec(a * x + b * y)
    e_lin = (torch.linalg.vector_norm(lin - (a * hx + b * hy)) / torch.linalg.vector_norm(lin)).item()
    # H is Hermitian on the subspace: <y, Hx> = <Hy, x>
    l, r = torch.vdot(y, hx).item(), torch.vdot(hy, x).item()
    e_herm = abs(l - r) / max(abs(l), 1e-300)
    assert e_lin < tol and e_herm < tol, (e_lin, e_herm)
    return hx


def test_hubbard_full_size_free_equals_conn_and_is_hermitian():
    """Hubbard 4x4, D = 2^20 (the headline workload): FREE (hash) and CONN products agree bit for
    bit, and the operator is linear and Hermitian to rounding."""
    import torch
    from rqutils_gb300 import workloads as W
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    h = PauliSumXZ.from_paulisum(W.hubbard_jw(4, 4, 1.0, 4.0), force_real=True, add_padding=True)
    S = W.sample_sector(np.random.default_rng(1), 1 << 20, [(16, 8), (16, 8)])
    terms = DeviceTerms(h)
    sub = DeviceSubspace(S, num_qubits=32)
    free = DeviceOperator(terms, sub, mode='free')
    conn = DeviceOperator(terms, sub, mode='conn')
    rng = np.random.default_rng(2)
    hx = _hermitian_checks(free, sub.D, torch.complex128, rng, 1e-12)
    x = torch.as_tensor(rng.normal(size=sub.D) + 1j * rng.normal(size=sub.D)).cuda()
    assert torch.equal(free.matvec(x), conn.matvec(x))
    free.check_errors()


def test_chemistry_2e24_rows_with_presence_bitmap():
    """64-qubit chemistry Hamiltonian (50,000 terms) on 2^24 states of the 16a/16b sector: the
    presence bitmap is built (table larger than L2), FREE and CONN agree, and the product is
    linear and Hermitian."""
    import torch
    from rqutils_gb300 import workloads as W
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    p, c = W.chemistry_jw(32, np.random.default_rng(4), keep=50000)
    h = PauliSumXZ.from_paulisum((p, c), force_real=True, add_padding=True)
    S = W.sample_sector(np.random.default_rng(5), 1 << 24, [(32, 16), (32, 16)])
    terms = DeviceTerms(h)
    sub = DeviceSubspace(S, num_qubits=64)
    assert sub.pbits > 0
    free = DeviceOperator(terms, sub, mode='free')
    rng = np.random.default_rng(6)
    _hermitian_checks(free, sub.D, torch.complex64, rng, 1e-5)
    conn = DeviceOperator(terms, sub, mode='conn')
    x = torch.as_tensor(rng.normal(size=sub.D) + 1j * rng.normal(size=sub.D)).to(torch.complex64).cuda()
    assert torch.equal(free.matvec(x), conn.matvec(x))
    free.check_errors()


def test_uniquify_2e26_samples():
    """2^26 raw samples with duplicates (the chemistry subspace size): sorted, distinct, and the
    same multiset of values (a checksum of the distinct values and their count)."""
    import torch
    from rqutils_gb300.sqd import uniquify_device
    rng = np.random.default_rng(7)
    base = rng.integers(0, 2 ** 62, size=(1 << 26) - (1 << 22), dtype=np.uint64)
    raw = np.concatenate([base, base[:1 << 22]])
    rng.shuffle(raw)
    t = torch.from_numpy(raw.view(np.int64)).cuda()
    out = uniquify_device(t)
    assert torch.all(out[1:] > out[:-1]).item()  # values below 2^62: signed order is unsigned order
    ref = np.unique(base)
    assert out.numel() == len(ref)
    got = out.cpu().numpy().view(np.uint64)
    assert int(np.bitwise_xor.reduce(got)) == int(np.bitwise_xor.reduce(ref))
    assert int((got % np.uint64(1000003)).sum()) == int((ref % np.uint64(1000003)).sum())
