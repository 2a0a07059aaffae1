"""``jax.lax`` stand-in: control flow run eagerly, stable multi-key sort via np.lexsort."""
import numpy as _np

from ._core import asjarray


class Precision:
    DEFAULT = 0
    HIGH = 1
    HIGHEST = 2


def _tree_index(xs, i):
    if isinstance(xs, (tuple, list)):
        return type(xs)(_tree_index(x, i) for x in xs)
    if isinstance(xs, dict):
        return {k: _tree_index(v, i) for k, v in xs.items()}
    if hasattr(type(xs), '_shim_data'):  # registered dataclass: slice the data fields
        kw = {k: _tree_index(getattr(xs, k), i) for k in type(xs)._shim_data}
        kw.update({k: getattr(xs, k) for k in type(xs)._shim_static})
        return type(xs)(**kw)
    return asjarray(_np.asarray(xs)[i])


def _tree_len(xs):
    if isinstance(xs, (tuple, list)):
        return _tree_len(xs[0])
    if isinstance(xs, dict):
        return _tree_len(next(iter(xs.values())))
    if hasattr(type(xs), '_shim_data'):
        return _tree_len(getattr(xs, type(xs)._shim_data[0]))
    return _np.asarray(xs).shape[0]


def _tree_stack(ys):
    first = ys[0]
    if first is None:
        return None
    if isinstance(first, (tuple, list)):
        return type(first)(_tree_stack([y[k] for y in ys]) for k in range(len(first)))
    if isinstance(first, dict):
        return {k: _tree_stack([y[k] for y in ys]) for k in first}
    return asjarray(_np.stack([_np.asarray(y) for y in ys]))


def scan(f, init, xs=None, length=None, **_kwargs):
    n = length if xs is None else _tree_len(xs)
    carry = init
    ys = []
    for i in range(n):
        carry, y = f(carry, None if xs is None else _tree_index(xs, i))
        ys.append(y)
    return carry, (_tree_stack(ys) if ys else None)


def while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def sort(operand, dimension=-1, is_stable=True, num_keys=1):
    if not isinstance(operand, (tuple, list)):
        return asjarray(_np.sort(_np.asarray(operand), axis=dimension, kind='stable'))
    ops = [_np.asarray(o) for o in operand]
    assert all(o.ndim == 1 for o in ops), 'only 1-d operands are supported'
    keys = ops[:num_keys]
    order = _np.lexsort(tuple(reversed(keys)))  # lexsort is stable, last key is primary
    return tuple(asjarray(o[order]) for o in ops)


def ne(x, y):
    return asjarray(_np.asarray(_np.not_equal(x, y)))


def iota(dtype, size):
    return asjarray(_np.arange(size, dtype=dtype))


def broadcasted_iota(dtype, shape, dimension, out_sharding=None):
    shape = tuple(shape)
    ar = _np.arange(shape[dimension], dtype=dtype)
    view = [1] * len(shape)
    view[dimension] = shape[dimension]
    return asjarray(_np.broadcast_to(ar.reshape(view), shape).copy())


def dot(a, b, precision=None, out_sharding=None, **_kwargs):
    return asjarray(_np.asarray(_np.dot(a, b)))
