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
