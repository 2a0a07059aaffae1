"""GB300-native SQD hot path of rqutils: Pauli-sum subspace matvec + single-vector LOBPCG.

Module layout mirrors rqutils: ``rqutils_gb300.sqd`` (``sqd``, ``hproj``),
``rqutils_gb300.ground_locg`` (``ground_locg``), ``rqutils_gb300.paulis.symplectic``
(``PauliSumXZ``).  Device objects live in ``rqutils_gb300.device``.  All device work runs in
``_lib/librqsqd.so`` (CUDA, sm_103a), built by ``python -m rqutils_gb300._build``.
"""
__version__ = '0.1.0'

from .paulis.symplectic import PauliSumXZ  # noqa: F401
