"""NumPy stand-in for the subset of the ``jax`` API that rqutils' SQD modules use.

This package exists only so that ``tests/golden/make_golden.py`` can import and run the
unmodified reference modules (``rqutils/sqd.py``, ``rqutils/ground_locg.py``,
``rqutils/paulis/symplectic.py``) in a container where jax is not installed, and record their
outputs as golden fixtures.  It is test infrastructure: nothing in the product imports it.

Semantics mirrored from jax (64-bit mode, single device):

* arrays are immutable: in-place operators return new arrays, ``x.at[idx].set/add/...`` copy;
* ``x.at[idx].get(mode='fill', fill_value=v, wrap_negative_indices=False)`` returns ``v``
  wherever an index is outside ``[0, size)``;
* ``jnp.bincount(x, length=L)`` drops values ``>= L``;
* ``jax.lax.sort`` is a stable lexicographic sort over the first ``num_keys`` operands;
* ``jit`` runs eagerly; sharding arguments are accepted and ignored (no mesh is ever set).
"""
import numpy as _np

from . import numpy, lax, sharding, tree_util, debug, tree  # noqa: F401
from ._core import JArray as Array, asjarray as _asj, jit, reshard, typeof  # noqa: F401


class _Config:
    def update(self, *_args, **_kwargs):
        pass


config = _Config()


def device_count():
    return 1


def set_mesh(_mesh):
    raise NotImplementedError('the NumPy stand-in runs on a single device only')
