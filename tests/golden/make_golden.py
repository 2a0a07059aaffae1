"""Generate golden fixtures by running the reference's own SQD code.

Run in a container that has the rqutils sources (read-only) but no jax:

    python tests/golden/make_golden.py /path/to/rqutils-checkout            # SQD cases
    python tests/golden/make_golden.py /path/to/rqutils-checkout --svsim    # svsim cases

The reference modules ``rqutils/paulis/symplectic.py``, ``rqutils/sqd.py`` and
``rqutils/ground_locg.py`` are imported unmodified; ``jax`` is provided by the NumPy stand-in in
``tests/golden/jaxshim`` (eager execution, 64-bit).  Package ``__init__`` files are bypassed
(they need installed metadata and unrelated modules).  Each case writes ``case_<name>.npz`` next
to this script with the inputs, the reference's intermediate arrays and its final outputs.

With ``--svsim`` the reference's state-vector simulator ``rqutils/svsim.py`` is imported the same
way and each circuit case writes ``svsim_<name>.npz``: the gate list, the reference's CircuitXZ
arrays (``to_circuitxz``), the initial state and the final state of ``svsim``.
"""
import os
import sys
import types
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(root):
    sys.path.insert(0, os.path.join(HERE, 'jaxshim'))
    for name, sub in (('rqutils', 'rqutils'), ('rqutils.paulis', 'rqutils/paulis')):
        mod = types.ModuleType(name)
        mod.__path__ = [os.path.join(root, sub)]
        sys.modules[name] = mod
    import rqutils.sqd as rsqd
    import rqutils.ground_locg as rlocg
    from rqutils.paulis.symplectic import PauliSumXZ
    return rsqd, rlocg, PauliSumXZ


def random_strings(rng, n, K, alphabet='IXYZ'):
    return [''.join(alphabet[i] for i in row) for row in rng.choice(len(alphabet), size=(K, n))]


def local_strings(rng, n, K, lo=1, hi=4):
    out = []
    for _ in range(K):
        w = int(rng.integers(lo, hi + 1))
        sup = rng.choice(n, size=w, replace=False)
        row = ['I'] * n
        for q in sup:
            row[n - 1 - q] = 'XYZ'[int(rng.integers(0, 3))]
        out.append(''.join(row))
    return out


def weight_states(rng, n, w, D):
    rows = np.zeros((D, n), dtype=np.uint8)
    seen = set()
    k = 0
    while k < D:
        cols = rng.choice(n, size=w, replace=False)
        key = tuple(sorted(cols))
        if key in seen:
            continue
        seen.add(key)
        rows[k, cols] = 1
        k += 1
    return rows


def hubbard_2x2():
    """Fermi-Hubbard 2x2, open boundary, t = 1, U = 4, 8 spin-orbitals (qubit i up, 4 + i down)."""
    n, Ns = 8, 4
    bonds = [(0, 1), (2, 3), (0, 2), (1, 3)]
    terms = {}

    def lab(ops):
        row = ['I'] * n
        for q, p in ops.items():
            row[n - 1 - q] = p
        return ''.join(row)

    def add(k, c):
        terms[k] = terms.get(k, 0.) + c

    for i, j in bonds:
        for off in (0, Ns):
            p, q = i + off, j + off
            chain = {k: 'Z' for k in range(p + 1, q)}
            add(lab({**chain, p: 'X', q: 'X'}), -0.5)
            add(lab({**chain, p: 'Y', q: 'Y'}), -0.5)
    for i in range(Ns):
        add(lab({}), 1.)
        add(lab({i: 'Z'}), -1.)
        add(lab({Ns + i: 'Z'}), -1.)
        add(lab({i: 'Z', Ns + i: 'Z'}), 1.)
    keys = sorted(terms)
    return keys, np.array([terms[k] for k in keys])


def build_cases():
    rng = np.random.default_rng(20261203)
    cases = {}
    # Small version of the reference notebook (tests/sqd.ipynb): random IXYZ strings, U(-1,1),
    # duplicate-heavy random 0/1 samples.
    n = 8
    cases['notebook'] = dict(paulis=random_strings(rng, n, 40), coeffs=rng.uniform(-1, 1, 40),
                             states=rng.choice(2, size=(300, n)).astype(np.uint8))
    # Benchmark-config-0 shape at a small D: locality 1..4, N(0,1), weight-n/2 subspace.
    n = 20
    cases['local20'] = dict(paulis=local_strings(rng, n, 200), coeffs=rng.normal(size=200),
                            states=weight_states(rng, n, 10, 600))
    # Real Hamiltonian (Fermi-Hubbard 2x2): float64 path.
    p, c = hubbard_2x2()
    rows = []
    for up in range(16):
        for dn in range(16):
            if bin(up).count('1') == 2 and bin(dn).count('1') == 2:
                s = up | (dn << 4)
                rows.append([(s >> (7 - col)) & 1 for col in range(8)])
    rows = np.array(rows, dtype=np.uint8)
    keep = rng.choice(len(rows), size=30, replace=False)
    cases['hubbard2x2'] = dict(paulis=p, coeffs=c, states=rows[keep])
    # Consolidation quirks: duplicates cancelling to an exact zero and a purely imaginary
    # coefficient (force_real makes it zero) both truncate their X group's diagonal loop.
    n = 6
    base = random_strings(rng, n, 30)
    extra = ['XXIIII', 'XXIIII', 'XXZIII', 'YYIIII', 'IIIIXZ', 'IIIIXZ', 'IIIIXI']
    coeffs = list(rng.uniform(-1, 1, 30)) + [0.5, -0.5, 0.7, -0.3, 0.25j, 0., 0.4]
    cases['zero_coeff'] = dict(paulis=base + extra, coeffs=np.array(coeffs),
                               states=rng.choice(2, size=(50, n)).astype(np.uint8))
    # states_size larger than the number of unique states: fill rows.
    n = 10
    cases['fill_rows'] = dict(paulis=random_strings(rng, n, 50), coeffs=rng.uniform(-1, 1, 50),
                              states=rng.choice(2, size=(150, n)).astype(np.uint8),
                              states_size=200)
    # No diagonal (x = 0) group: initial vector is one-hot at index 0.
    n = 9
    nd = [s for s in random_strings(rng, n, 80, 'IXY') if set(s) & {'X', 'Y'}][:40]
    cases['no_diag'] = dict(paulis=nd, coeffs=rng.uniform(-1, 1, len(nd)),
                            states=rng.choice(2, size=(120, n)).astype(np.uint8))
    # n a multiple of 8 (the padding bit makes B = n/8 + 1).
    n = 16
    cases['n16'] = dict(paulis=local_strings(rng, n, 60), coeffs=rng.normal(size=60),
                        states=weight_states(rng, n, 8, 400))
    # The two cases above start from an isolated state (an exact eigenvector with zero residual),
    # where the reference's 2x2 Rayleigh-Ritz divides by zero and its result is NaN after maxiter
    # iterations.  Converging cases of the same shape use a well-filled weight sector instead.
    n = 12
    cases['local12'] = dict(paulis=local_strings(rng, n, 150), coeffs=rng.normal(size=150),
                            states=weight_states(rng, n, 6, 600))
    n = 16
    cases['n16dense'] = dict(paulis=local_strings(rng, n, 80), coeffs=rng.normal(size=80),
                             states=rng.choice(2, size=(2500, n)).astype(np.uint8))
    return cases


def run_case(rsqd, rlocg, PauliSumXZ, case, rng):
    paulis, coeffs, states = case['paulis'], np.asarray(case['coeffs']), case['states']
    states_size = case.get('states_size', states.shape[0])
    out = dict(paulis=np.array(paulis), coeffs=coeffs, states=states,
               states_size=np.int64(states_size))
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        ham = PauliSumXZ.from_paulisum((paulis, coeffs), force_real=True, add_padding=True)
        ham_nopad = PauliSumXZ.from_paulisum((paulis, coeffs))
    out.update(ham_x=np.asarray(ham.x), ham_z=np.asarray(ham.z), ham_c=np.asarray(ham.c),
               nopad_x=np.asarray(ham_nopad.x), nopad_z=np.asarray(ham_nopad.z),
               nopad_c=np.asarray(ham_nopad.c), num_qubits=np.int64(ham.num_qubits))
    states_p = np.packbits(np.pad(states.astype(np.uint8), {1: (1, 0)}), axis=1)
    states_u = np.asarray(rsqd.uniquify_states(states_p, states_size))
    D = int(np.searchsorted(states_u[:, 0] >> 7, 1))
    xs = np.stack([np.asarray(rsqd.get_xsource(xj, states_u)) for xj in ham.x]).astype(np.int32)
    diags = np.stack([np.asarray(rsqd.get_diagonal(zj, cj, states_u))
                      for zj, cj in zip(ham.z, ham.c)])
    vecs = rng.normal(size=(2, states_size)) + 1j * rng.normal(size=(2, states_size))
    vecs[:, D:] = 0
    if np.isrealobj(ham.c):
        vecs = vecs.real.copy()
    mv = np.stack([np.asarray(rsqd.apply_h_x_cached(v, xs, ham.z, ham.c, states_u))
                   for v in vecs])
    out.update(states_u=states_u, D=np.int64(D), xsources=xs, diagonals=diags, mv_in=vecs,
               mv_out=mv)

    record = {}
    original = rsqd.ground_locg

    def recording(matvec, vinit, args=(), **kw):
        record['vinit'] = np.asarray(vinit)
        res = original(matvec, vinit, args=args, **kw)
        record['niter'] = int(res[2])
        return res

    rsqd.ground_locg = recording
    try:
        eigval, eigvec, basis = rsqd.sqd((paulis, coeffs), states, states_size=states_size)
    finally:
        rsqd.ground_locg = original
    out.update(eigval=np.float64(eigval), eigvec=np.asarray(eigvec), basis=np.asarray(basis),
               vinit=record['vinit'], niter=np.int64(record['niter']))
    return out


def fullspace_case(PauliSumXZ, rng):
    n = 6
    paulis = random_strings(rng, n, 30)
    coeffs = rng.uniform(-1, 1, 30) + 1j * rng.uniform(-1, 1, 30)
    ham = PauliSumXZ.from_paulisum((paulis, coeffs))
    from jax import Array as JaxArray  # the stand-in's array type (matmul is not jitted)
    rhs1 = (rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)).view(JaxArray)
    return dict(paulis=np.array(paulis), coeffs=coeffs, ham_x=np.asarray(ham.x),
                ham_z=np.asarray(ham.z), ham_c=np.asarray(ham.c), num_qubits=np.int64(n),
                rhs1=np.asarray(rhs1), out1=np.asarray(ham.matmul(rhs1)))
    # (A 2-d right-hand side fails inside the reference's own expand_dims call,
    # symplectic.py:146, so only the 1-d form is recorded.)


def svsim_cases():
    """Random circuits of every gate kind the reference accepts in a gate list (x, y, z, rx, ry,
    rz, rzz), one-hot and dense initial states, angles including 0 and +-2 pi."""
    rng = np.random.default_rng(20261204)
    names = ['x', 'y', 'z', 'rx', 'ry', 'rz', 'rzz']

    def circuit(n, ngates, angles=None):
        out = []
        for _ in range(ngates):
            nm = names[rng.integers(len(names))]
            if nm == 'rzz':
                q = [int(v) for v in rng.choice(n, size=2, replace=False)]
            else:
                q = int(rng.integers(n))
            if nm.startswith('r'):
                th = float(rng.uniform(-np.pi, np.pi)) if angles is None else float(rng.choice(angles))
                out.append((nm, q, th))
            else:
                out.append((nm, q))
        return out

    dense8 = rng.normal(size=256) + 1j * rng.normal(size=256)
    return {
        'mixed6': (circuit(6, 40), 5),
        'dense8': (circuit(8, 60), dense8 / np.linalg.norm(dense8)),
        'edge5': (circuit(5, 30, angles=[0., 2 * np.pi, -2 * np.pi, np.pi, -np.pi / 2]) +
                  [('rx', 4, 0.3), ('x', 4), ('rzz', [0, 4], 1.1)], 0),
        'deep10': (circuit(10, 200), 1023),
    }


def run_svsim_case(rsv, circ, init):
    names = np.array([g[0] for g in circ])
    qubits = np.full((len(circ), 2), -1, dtype=np.int64)
    angles = np.zeros(len(circ))
    for k, g in enumerate(circ):
        q = np.atleast_1d(np.asarray(g[1], dtype=np.int64))
        qubits[k, :len(q)] = q
        if len(g) > 2:
            angles[k] = g[2]
    cxz = rsv.to_circuitxz(circ)
    init_arg = np.int64(init) if np.ndim(init) == 0 else np.asarray(init, dtype=np.complex128)
    final = np.asarray(rsv.svsim(circ, init_arg))
    return dict(names=names, qubits=qubits, angles=angles, x=np.asarray(cxz.x),
                z=np.asarray(cxz.z), cos=np.asarray(cxz.cos), sin=np.asarray(cxz.sin),
                num_qubits=np.int64(cxz.num_qubits), initial=np.asarray(init_arg), final=final)


def main_svsim(root):
    load_reference(root)
    import rqutils.svsim as rsv
    for name, (circ, init) in svsim_cases().items():
        data = run_svsim_case(rsv, circ, init)
        np.savez_compressed(os.path.join(HERE, f'svsim_{name}.npz'), **data)
        print(f'svsim {name}: n={int(data["num_qubits"])} gates={len(circ)} '
              f'|psi|={np.linalg.norm(data["final"]):.15f}')


def main():
    args = [a for a in sys.argv[1:] if not a.startswith('--')]
    root = args[0] if args else os.environ.get('RQUTILS_REFERENCE')
    if not root or not os.path.isdir(os.path.join(root, 'rqutils')):
        raise SystemExit('usage: make_golden.py <rqutils checkout> [--svsim]')
    if '--svsim' in sys.argv:
        main_svsim(root)
        return
    rsqd, rlocg, PauliSumXZ = load_reference(root)
    rng = np.random.default_rng(7)
    for name, case in build_cases().items():
        data = run_case(rsqd, rlocg, PauliSumXZ, case, rng)
        np.savez_compressed(os.path.join(HERE, f'case_{name}.npz'), **data)
        print(f'{name}: J={data["ham_x"].shape[0]} D={int(data["D"])} '
              f'eig={float(data["eigval"]):.12f} niter={int(data["niter"])}')
    data = fullspace_case(PauliSumXZ, rng)
    np.savez_compressed(os.path.join(HERE, 'case_fullspace.npz'), **data)
    print('fullspace: ok')


if __name__ == '__main__':
    main()
