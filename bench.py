"""Benchmark of the SQD hot path on one GB300.

Workload (the configuration the headline metric is quoted on): Fermi-Hubbard 4x4, periodic,
t = 1, U = 4, Jordan-Wigner mapped to 32 qubits (65 X groups, 177 terms after consolidation);
subspace of D = 2^20 bitstrings drawn uniformly without replacement from the 8-up / 8-down sector
(seed 1); complex64 vectors with FP32 compensated accumulation.

A step is one matrix-free Pauli-sum matvec y = H x over the whole subspace (hash lookups, the
reference's cache_level (0, *) path) with x resident in HBM.  Between timed steps a 256 MiB buffer
is written to flush the 129 MB L2 (the working set, ~56 MB, would otherwise stay L2-resident); each
step is timed with CUDA events on the launching stream.  ``e2e`` times the same step through the
public API with the input copied from pinned host memory and the output copied back inside the
timed region.  Extra keys: cached-connectivity and CSR matvec rates, LOBPCG time to a relative
residual of 1e-8, the roofline of the matvec kernel and the CPU baseline (the oracle's restatement
of the reference's matvec, timed on the host cores on a bounded sample).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'Pauli-matvec/s & time-to-residual 1e-8 (learned warm-start vs plain), 1 GB300'
UNIT = 'matvec/s'
D_BENCH = 1 << 20
SEED = 1
L2_FLUSH_BYTES = 256 << 20
PROFILE_TRAFFIC = os.path.join(ROOT, 'profiles', 'matvec_free_hubbard4x4_D1048576.txt')


def workload():
    from rqutils_gb300 import workloads
    from rqutils_gb300.paulis.symplectic import PauliSumXZ
    p, c = workloads.hubbard_jw(4, 4, 1.0, 4.0, periodic=True)
    ham = PauliSumXZ.from_paulisum((p, c), force_real=True, add_padding=True)
    rng = np.random.default_rng(SEED)
    S = workloads.sample_sector(rng, D_BENCH, [(16, 8), (16, 8)])
    x = workloads.random_vector(np.random.default_rng(SEED + 1), D_BENCH, complex_=True)
    return ham, S, x


def config(extra=None):
    cfg = {'workload': 'hubbard4x4_periodic_t1_U4_jw32_D1048576_sector8u8d',
           'D': D_BENCH, 'num_qubits': 32, 'groups': 65, 'terms': 177,
           'matvec_mode': 'matrix-free (hash lookup, sector filter)',
           'l2_policy': 'flush 256 MiB between timed steps', 'seed': SEED}
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.index}', f'--query-gpu={self.QUERY}',
                 '--format=csv,noheader,nounits', '-lms', '20'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [v.strip() for v in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(name)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': smax,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------------------------------------
# distributed helpers (replicas only: every rank runs the same single-GPU workload)
# ---------------------------------------------------------------------------------------------
def dist_init():
    import torch
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
        dist.init_process_group('nccl')
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device='cuda')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------------------------
def algorithmic_bytes(D, J, J0, hits, bv):
    """Bytes of one matvec: states (8 D) + x[i] for the diagonal group (bv D) + y (bv D) + one
    8-byte key probe per off-diagonal lookup (8 D (J - J0)) + the gathered source amplitudes
    (bv hits); term tables are negligible."""
    return 8 * D + bv * D + bv * D + 8 * D * (J - J0) + bv * hits


def read_profile_traffic():
    try:
        with open(PROFILE_TRAFFIC) as fh:
            for line in fh:
                if line.startswith('dram_bytes_per_launch:'):
                    return float(line.split(':', 1)[1])
    except OSError:
        pass
    return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            p = json.load(fh)
        return float(p['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def time_steps(fn, steps, flush, stream):
    """Per-step CUDA-event durations (ms) of fn(), with the L2 flushed before every step."""
    import torch
    evs = []
    for _ in range(steps):
        flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def run_ours(args, rank, ws):
    import torch
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    from rqutils_gb300.ground_locg import lobpcg_solve

    dev = torch.device('cuda', torch.cuda.current_device())
    ham, S, xh = workload()
    terms = DeviceTerms(ham, device=dev)
    sub = DeviceSubspace(S, num_qubits=32, device=dev)
    op_free = DeviceOperator(terms, sub, mode='free')
    op_conn = DeviceOperator(terms, sub, mode='conn')
    op_csr = DeviceOperator(terms, sub, mode='csr', csr_vtype=2)
    hits = op_conn.nnz
    D, J, J0 = sub.D, terms.J, 1 if terms.diag_group >= 0 else 0
    x = torch.as_tensor(xh).to(dev, torch.complex64)
    y = torch.empty_like(x)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def flush():
        flush_buf.fill_(1.0)

    def mv_free():
        op_free.matvec(x, out=y)

    clk = ClockSampler(index=torch.cuda.current_device()).__enter__()
    for _ in range(args.warmup):
        mv_free()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    times = time_steps(mv_free, args.steps, flush, stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier(ws)
    op_free.check_errors()
    t_step = max_over_ranks(sum(times) / 1e3, ws)  # seconds for K steps, max over ranks
    value = ws * args.steps / t_step
    ms_per_step = 1e3 * t_step / args.steps

    # parity spot check of the timed output against the cached-connectivity path
    y_conn = op_conn.matvec(x)
    rel = float(torch.linalg.vector_norm(y - y_conn) / torch.linalg.vector_norm(y_conn))

    # other modes (same flush policy)
    for op in (op_conn, op_csr):
        for _ in range(args.warmup):
            op.matvec(x, out=y)
    t_conn = statistics.mean(time_steps(lambda: op_conn.matvec(x, out=y), args.steps, flush, stream))
    t_csr = statistics.mean(time_steps(lambda: op_csr.matvec(x, out=y), args.steps, flush, stream))
    # matrix-free without the sector filter (every off-diagonal lookup probes the table)
    sub_nf = DeviceSubspace(S, num_qubits=32, device=dev, filter_masks=(0, 0))
    op_nf = DeviceOperator(terms, sub_nf, mode='free')
    for _ in range(args.warmup):
        op_nf.matvec(x, out=y)
    t_nf = statistics.mean(time_steps(lambda: op_nf.matvec(x, out=y), args.steps, flush, stream))

    # e2e through the public API with host buffers
    xh_pin = torch.as_tensor(xh.astype(np.complex64)).pin_memory()
    yh_pin = torch.empty_like(xh_pin).pin_memory()
    xd = torch.empty_like(x)

    def e2e_step():
        xd.copy_(xh_pin, non_blocking=True)
        op_free.matvec(xd, out=y)
        yh_pin.copy_(y, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    e2e_times = time_steps(e2e_step, args.steps, flush, stream)
    clk.__exit__(None, None, None)
    e2e_t = max_over_ranks(sum(e2e_times) / 1e3, ws)
    e2e_value = ws * args.steps / e2e_t

    # roofline of the matvec kernel
    bv = 8
    abytes = algorithmic_bytes(D, J, J0, hits, bv)
    peak, peak_kind = measured_peaks()
    achieved = abytes / (ms_per_step / 1e3) / 1e9
    traffic = read_profile_traffic()

    # LOBPCG time to a relative residual of 1e-8 from a seeded random start.  (The reference's
    # one-hot start at the lowest diagonal entry is an isolated state of this subspace -- an exact
    # eigenvector with zero residual -- on which its Rayleigh-Ritz step breaks down.)
    lob = {}
    xr = np.random.default_rng(SEED + 2).normal(size=D)
    for name, kw in (('mixed_fast', dict(mixed=True, variant='fast')),
                     ('fp64_fast', dict(mixed=False, variant='fast')),
                     ('fp64_reference', dict(mixed=False, variant='reference'))):
        x0 = torch.as_tensor(xr, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eig, xs, info = lobpcg_solve(op_conn, x0, maxiter=3000, target_rel=1e-8, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # certify: FP64 residual with a fresh FP64 matvec
        ax = op_conn.matvec(xs)
        r = float(torch.linalg.vector_norm(ax - eig * xs))
        lob[name] = {'start': 'random (seeded)', 'time_s': round(dt, 4), 'iterations': info['niter'],
                     'iterations_32bit': info['niter_lo'], 'eigval': eig,
                     'rel_residual_fp64': r / abs(eig), 'converged': info['converged']}

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_per_step, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c64', 'data': 'synthetic',
        'config': config({'parallelism': f'replicas{ws}' if ws > 1 else 'single',
                          'hits_per_matvec': hits, 'wall_s_timed_region': round(wall, 3)}),
        'e2e': {'value': e2e_value, 'unit': UNIT, 'h2d_bytes_per_step': 8 * D,
                'd2h_bytes_per_step': 8 * D},
        'gpu_launches': args.steps,
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': traffic,
                     'peak_source': f'{peak_kind} hbm_gbs',
                     'algorithmic_bytes_per_launch': abytes},
        'modes': {'conn_matvec_per_s': 1e3 / t_conn, 'csr_matvec_per_s': 1e3 / t_csr,
                  'free_nofilter_matvec_per_s': 1e3 / t_nf,
                  'free_vs_conn_rel_diff': rel},
        'lobpcg': lob,
        'clocks': clk.summary(),
    }
    if rank == 0:
        line['cpu_baseline'] = cpu_baseline(ham, S, xh, steps=6)
        print(json.dumps(line), flush=True)


def run_profile(args):
    """Only the timed loop of the headline (warm-up, then flush + matvec per step): the command
    that the ncu launch list and the kernel capture are taken on."""
    import torch
    from rqutils_gb300.device import DeviceOperator, DeviceSubspace, DeviceTerms
    dev = torch.device('cuda', torch.cuda.current_device())
    ham, S, xh = workload()
    terms = DeviceTerms(ham, device=dev)
    sub = DeviceSubspace(S, num_qubits=32, device=dev)
    op = DeviceOperator(terms, sub, mode='free')
    x = torch.as_tensor(xh).to(dev, torch.complex64)
    y = torch.empty_like(x)
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        op.matvec(x, out=y)
    times = time_steps(lambda: op.matvec(x, out=y), args.steps,
                       lambda: flush_buf.fill_(1.0), torch.cuda.current_stream())
    op.check_errors()
    print(json.dumps({'profile_steps': args.steps, 'ms': times}), flush=True)


# ---------------------------------------------------------------------------------------------
# CPU baseline / reference arm: the oracle's restatement of the reference matvec
# ---------------------------------------------------------------------------------------------
def _oracle_setup(ham, S):
    from oracle.paulis import OracleTerms
    J = len(ham.xmask)
    counts = np.diff(ham.toff)
    kmax = int(counts.max())
    z = np.zeros((J, kmax), np.uint64)
    c = np.zeros((J, kmax), ham.coef.dtype)
    for j in range(J):
        a, b = ham.toff[j], ham.toff[j + 1]
        z[j, :b - a] = ham.zmask[a:b]
        c[j, :b - a] = ham.coef[a:b]
    return OracleTerms(x=ham.xmask.copy(), z=z, c=c, counts=counts, num_qubits=ham.num_qubits)


def cpu_baseline(ham, S, xh, steps=1):
    """apply_h (sqd.py:590-605, X sources re-derived by sort-merge every matvec) restated in
    NumPy, on all host cores (groups split over a thread pool), for `steps` full matvecs."""
    from oracle.sqd import matvec_nocache
    terms = _oracle_setup(ham, S)
    cores = os.cpu_count() or 1
    x = xh.astype(np.complex128)
    t0 = time.perf_counter()
    for _ in range(steps):
        matvec_nocache(x, terms, S, threads=cores)
    dt = time.perf_counter() - t0
    return {'value': steps / dt, 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'sample': f'{steps} full matvec(s) over the whole workload (D=2^20, 65 groups), '
                      'complex128, NumPy restatement of apply_h with per-group sort-merge'}


def run_reference(args, rank, ws):
    if rank != 0:
        return
    ham, S, xh = workload()
    # bounded sample: each step is one full matvec (~1-2 s on all host cores)
    steps = max(1, min(args.steps, 10))
    for _ in range(min(args.warmup, 1)):
        cpu_baseline(ham, S, xh, steps=1)
    cb = cpu_baseline(ham, S, xh, steps=steps)
    v = cb['value']
    print(json.dumps({
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': ws,
        'steps': steps, 'warmup': args.warmup, 'ms_per_step': 1e3 / v, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'c128', 'data': 'synthetic',
        'config': config({'note': 'reference JAX path not installable here (no jax); the '
                                  'NumPy restatement of its algorithm is timed'}),
        'cpu_baseline': cb,
        'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--profile', action='store_true',
                    help='run only the timed matvec loop (for ncu captures)')
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == 'ours':
        args.warmup = 3
    if args.impl == 'reference':
        rank = int(os.environ.get('RANK', '0'))
        run_reference(args, rank, int(os.environ.get('WORLD_SIZE', '1')))
        return
    from rqutils_gb300._build import build
    build()
    if args.profile:
        run_profile(args)
        return
    rank, ws = dist_init()
    run_ours(args, rank, ws)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
