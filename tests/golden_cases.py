"""Loader for the golden fixtures produced by tests/golden/make_golden.py."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def case_names():
    names = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, 'case_*.npz')))
    return [n for n in names if n != 'fullspace']


def load(name):
    with np.load(os.path.join(GOLDEN, f'case_{name}.npz'), allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


def packed_to_u64(packed, n, padded=True):
    """Reference packed rows (big-endian bytes, optional leading padding bit) -> uint64."""
    ncol = n + (1 if padded else 0)
    bits = np.unpackbits(np.asarray(packed, dtype=np.uint8), axis=-1)[..., :ncol]
    out = np.zeros(bits.shape[:-1], dtype=np.uint64)
    for q in range(n):
        out |= bits[..., ncol - 1 - q].astype(np.uint64) << np.uint64(q)
    return out


def hamiltonian(case):
    return [str(p) for p in case['paulis']], case['coeffs']


def svsim_case_names():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, 'svsim_*.npz')))


def load_svsim(name):
    """A state-vector fixture recorded from the reference's rqutils/svsim.py, with its gate list
    rebuilt as (name, qubit(s)[, angle]) specifiers."""
    d = dict(np.load(os.path.join(GOLDEN, f'svsim_{name}.npz'), allow_pickle=False))
    circ = []
    for nm, q, th in zip(d['names'], d['qubits'], d['angles']):
        nm = str(nm)
        qq = [int(v) for v in q if v >= 0]
        qarg = qq if nm == 'rzz' else qq[0]
        circ.append((nm, qarg, float(th)) if nm.startswith('r') else (nm, qarg))
    d['circuit'] = circ
    return d
