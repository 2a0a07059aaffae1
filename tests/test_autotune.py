"""The matvec-form autotuner: problem classes and the recorded choices (CPU), and the measured
choice on the device, whose operator gives the cached-connectivity product (GPU)."""
import json

import numpy as np
import pytest


def test_problem_class_and_cache_round_trip(tmp_path):
    import torch
    from rqutils_gb300.autotune import TuneCache, form_key, form_of, problem_class
    a = problem_class('one', 32, 1 << 20, 65, torch.complex64)
    assert a == 'one:n32:k32:d20:j6:complex64'
    assert problem_class('one', 33, 1 << 20, 65, torch.complex64).split(':')[2] == 'k64'
    assert problem_class('one', 32, 3 << 19, 65, torch.complex64) != a   # log2(D) rounds to 21
    f = ('free', 'hash', 9)
    assert form_of(form_key(f)) == f
    path = str(tmp_path / 'tune.json')
    c = TuneCache(path)
    assert c.get(a) is None
    c.put(a, f, {f: 0.5, ('conn', 'hash', 8): 0.7})
    assert c.get(a) == f
    with open(path) as fh:
        rec = json.load(fh)
    assert rec[a]['form'] == 'free/hash/9' and rec[a]['times']['conn/hash/8'] == 0.7
    assert TuneCache(path).get(a) == f           # read back by a new cache


@pytest.mark.gpu
def test_tuned_operator_gives_the_cached_product():
    import torch
    from rqutils_gb300 import workloads
    from rqutils_gb300.autotune import FORMS, TuneCache, tune
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    from rqutils_gb300.sqd import SQDProblem
    from rqutils_gb300._build import build
    build()
    rng = np.random.default_rng(91)
    labels, coeffs = workloads.random_pauli_sum(rng, 20, 200)
    S = workloads.sample_sector(rng, 16384, [(20, 10)])
    h = PauliSumXZ.from_paulisum((labels, coeffs), force_real=True, add_padding=True)
    cache = TuneCache()
    best, times = tune(h, S, cache=cache)
    assert best in FORMS and best in times and len(times) >= 5
    assert times[best] == min(times.values())
    again, t2 = tune(h, S, cache=cache)
    assert again == best and t2 == {}            # recorded: no second measurement
    auto = SQDProblem(h, S, cache_level='auto', tune_cache=cache)
    conn = SQDProblem(h, S, cache_level=(1, 0))
    x = torch.as_tensor(workloads.random_vector(rng, len(S))).cuda()
    ya, yc = auto.op.matvec(x), conn.op.matvec(x)
    assert (torch.linalg.vector_norm(ya - yc) / torch.linalg.vector_norm(yc)).item() <= 1e-12


@pytest.mark.gpu
def test_tuned_batch_solves_like_the_fixed_forms():
    import torch
    from rqutils_gb300.autotune import TuneCache
    from rqutils_gb300.batch import BatchedSQD
    from rqutils_gb300.workloads import batched_random_problems
    from rqutils_gb300._build import build
    build()
    hams, states, ns = batched_random_problems(92, P=12, n_range=(10, 24), k_range=(20, 200),
                                               d_range=(64, 4096))
    cache = TuneCache()
    b = BatchedSQD(hams, states, cache_level='auto', tune_cache=cache)
    assert b.mode in ('free', 'conn') and len(cache.records) == 1
    # three candidates: matrix-free with the line filter or the presence bitmap, connectivity
    assert len(next(iter(cache.records.values()))['times']) == 3
    ref = BatchedSQD(hams, states, cache_level=(1, 0))
    rng = np.random.default_rng(93)
    xr = rng.normal(size=b.D) + 1j * rng.normal(size=b.D)
    x0 = torch.as_tensor(xr.real if b.is_real else xr).to(b.dtype).cuda()
    e1, _, i1 = b.solve(x0=x0, variant='fast')
    e2, _, i2 = ref.solve(x0=x0, variant='fast')
    for p in range(b.P):
        if np.isnan(e2[p]):
            continue
        assert abs(e1[p] - e2[p]) <= 1e-10 * max(1., abs(e2[p])), p
