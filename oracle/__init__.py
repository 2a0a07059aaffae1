"""CPU oracle for the SQD hot path of rqutils 0.2.0 -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy (float64 / complex128), the reference algorithm of

* ``rqutils/paulis/symplectic.py`` -- Pauli-sum grouping by X signature and phasing;
* ``rqutils/sqd.py``                -- sorted subspace, X-source connectivity, diagonals,
                                       the default ``cache_level=(1, 0)`` matvec, the initial vector;
* ``rqutils/ground_locg.py``        -- the single-vector LOBPCG loop with its analytic 2x2 / 3x3
                                       Rayleigh-Ritz solves.

It is the checker for the CUDA implementation in ``rqutils_gb300`` and the CPU baseline that
``bench.py`` times.  Only the test suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm may import it; the product never does.

Parity pin.  The reference ships no golden vectors (its only SQD test, ``tests/sqd.ipynb`` cell 3,
compares ``sqd()`` with a dense ``eigh`` of the projected matrix and stores no outputs).  The
fixtures in ``tests/golden/*.npz`` were produced by running the reference's own ``sqd.py``,
``ground_locg.py`` and ``symplectic.py`` unmodified, with jax replaced by a NumPy stand-in
(``tests/golden/jaxshim``), by ``tests/golden/make_golden.py``.  ``tests/test_oracle_golden.py``
checks this oracle against them: connectivity tables bit-exact, diagonals / matvecs / LOBPCG
iterates to round-off, iteration counts exactly.  The notebook's dense-``eigh`` acceptance check is
restated in ``oracle/dense.py`` and applied as well.

Bit convention used throughout: a basis state is a ``uint64`` whose bit ``q`` is qubit ``q``;
character 0 of a Pauli string (and column 0 of a 0/1 state row) is qubit ``n-1``.  Sorting these
integers gives the same order as the reference's lexicographic sort of big-endian packed bytes with
a leading zero padding bit (``sqd.py:233-237``).
"""
