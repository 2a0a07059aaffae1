"""Device sample front end (rq_pack_states, rq_uniquify) against NumPy pack + unique."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module', autouse=True)
def built():
    from rqutils_gb300._build import build
    build()


def _uniq(a):
    import torch
    from rqutils_gb300.sqd import uniquify_device
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()
    before = t.clone()
    out = uniquify_device(t).cpu().numpy().view(np.uint64)
    assert torch.equal(t, before)  # input untouched
    return out


@pytest.mark.parametrize('case', ['random64', 'dups32', 'one', 'equal', 'sorted', 'reversed',
                                  'top_bit', 'ragged', 'low_byte_only', 'large'])
def test_uniquify_matches_numpy(case):
    rng = np.random.default_rng(sum(map(ord, case)))
    if case == 'random64':
        a = rng.integers(0, 2**63, size=100000, dtype=np.uint64) * np.uint64(2) + np.uint64(1)
        a = np.concatenate([a, a[:5000]])
        rng.shuffle(a)
    elif case == 'dups32':
        a = rng.integers(0, 50000, size=200000).astype(np.uint64)
    elif case == 'one':
        a = np.array([12345], np.uint64)
    elif case == 'equal':
        a = np.full(5000, 0xDEADBEEF, np.uint64)
    elif case == 'sorted':
        a = np.arange(70000, dtype=np.uint64) * np.uint64(3)
    elif case == 'reversed':
        a = (np.arange(70000, dtype=np.uint64) * np.uint64(7))[::-1].copy()
    elif case == 'top_bit':
        a = rng.integers(0, 1000, size=30000).astype(np.uint64) | np.uint64(1 << 63)
        a[::7] = np.uint64(0xFFFFFFFFFFFFFFFF)
        a[::11] = np.uint64(0)
    elif case == 'ragged':
        a = rng.integers(0, 2**40, size=4096 * 3 + 17, dtype=np.uint64)
    elif case == 'low_byte_only':
        a = (np.uint64(0xABCD000000000000) | rng.integers(0, 256, size=9999).astype(np.uint64))
    else:
        a = rng.integers(0, 2**34, size=3_000_000, dtype=np.uint64)
    np.testing.assert_array_equal(_uniq(a), np.unique(a))


@pytest.mark.parametrize('n', [1, 7, 32, 40, 64])
def test_pack_matches_host(n):
    from rqutils_gb300.sqd import pack_states, pack_states_device
    rng = np.random.default_rng(n)
    bits = rng.integers(0, 2, size=(3000, n)).astype(np.uint8)
    got = pack_states_device(bits).cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(got, pack_states(bits))


def test_device_front_end_matches_reference_fixture_basis():
    """The reference fixtures' deduplicated bases come out of the device front end."""
    from golden_cases import case_names, load
    from rqutils_gb300.sqd import subspace_states_device, unpack_states
    for name in case_names():
        c = load(name)
        n = int(c['num_qubits'])
        _, S = subspace_states_device(c['states'], n)
        np.testing.assert_array_equal(unpack_states(S, n), c['basis'])
