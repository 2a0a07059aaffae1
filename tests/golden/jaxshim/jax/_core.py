"""Array type and transformation stubs for the NumPy stand-in of jax."""
import functools
import numpy as np


class JArray(np.ndarray):
    """ndarray with jax's functional ``.at`` updates and non-mutating in-place operators."""

    @property
    def at(self):
        return _AtIndexer(self)

    def __iter__(self):
        for i in range(self.shape[0]):
            yield super().__getitem__(i)

    def __getitem__(self, idx):
        # jax clamps out-of-range scalar integer indices instead of raising
        if isinstance(idx, (int, np.integer)) and self.ndim >= 1:
            n = self.shape[0]
            idx = min(max(int(idx), -n), n - 1)
        elif isinstance(idx, tuple):
            idx = tuple(
                min(max(int(i), -self.shape[k]), self.shape[k] - 1)
                if isinstance(i, (int, np.integer)) and k < self.ndim else i
                for k, i in enumerate(idx))
        return super().__getitem__(idx)

    # jax arrays are immutable: ``a -= b`` rebinds ``a`` instead of writing into the buffer
    def __iadd__(self, other):
        return self + other

    def __isub__(self, other):
        return self - other

    def __imul__(self, other):
        return self * other

    def __itruediv__(self, other):
        return self / other


def asjarray(obj):
    """Convert ndarrays (also inside tuples/lists) to JArray views; leave everything else."""
    if isinstance(obj, JArray):
        return obj
    if isinstance(obj, np.ndarray):
        return obj.view(JArray)
    if isinstance(obj, tuple):
        return tuple(asjarray(o) for o in obj)
    if isinstance(obj, list):
        return [asjarray(o) for o in obj]
    return obj


class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtRef(self._arr, idx)


class _AtRef:
    def __init__(self, arr, idx):
        self._arr = np.asarray(arr)
        self._idx = idx if isinstance(idx, tuple) else (idx,)

    def _expanded(self):
        """Index tuple with Ellipsis expanded, so that each entry maps to one array axis."""
        idx = self._idx
        if any(i is Ellipsis for i in idx):
            pos = next(k for k, i in enumerate(idx) if i is Ellipsis)
            nfill = self._arr.ndim - (len(idx) - 1)
            idx = idx[:pos] + (slice(None),) * nfill + idx[pos + 1:]
        return idx

    def get(self, mode=None, fill_value=None, wrap_negative_indices=True, out_sharding=None,
            **_kwargs):
        idx = self._expanded()
        arr = self._arr
        if mode != 'fill':
            return asjarray(np.asarray(arr[idx]))
        # Exactly one integer-array index is used by the reference modules.
        axes = [k for k, i in enumerate(idx) if isinstance(i, np.ndarray)]
        assert len(axes) == 1, 'fill-mode gather supports a single array index'
        axis = axes[0]
        ind = np.asarray(idx[axis]).astype(np.int64)
        size = arr.shape[axis]
        if wrap_negative_indices:
            ind = np.where(ind < 0, ind + size, ind)
        valid = (ind >= 0) & (ind < size)
        safe = np.where(valid, ind, 0)
        new_idx = idx[:axis] + (safe,) + idx[axis + 1:]
        out = arr[new_idx]
        mask = valid.reshape((1,) * axis + valid.shape + (1,) * (arr.ndim - axis - 1))
        fill = np.array(fill_value if fill_value is not None else 0, dtype=arr.dtype)
        return asjarray(np.where(mask, out, fill).astype(arr.dtype))

    def _update(self, op, value):
        out = np.array(self._arr, copy=True)
        idx = self._expanded()
        if op == 'set':
            out[idx] = value
        elif op == 'add':
            out[idx] = out[idx] + value
        elif op == 'subtract':
            out[idx] = out[idx] - value
        elif op == 'multiply':
            out[idx] = out[idx] * value
        return asjarray(out)

    def set(self, value, **_kwargs):
        return self._update('set', value)

    def add(self, value, **_kwargs):
        return self._update('add', value)

    def subtract(self, value, **_kwargs):
        return self._update('subtract', value)

    def multiply(self, value, **_kwargs):
        return self._update('multiply', value)


def jit(fun=None, **_kwargs):
    """Eager stand-in for jax.jit: converts array arguments to JArray and calls the function."""
    if fun is None:
        return lambda f: jit(f)

    @functools.wraps(fun)
    def wrapper(*args, **kwargs):
        args = asjarray(args)
        kwargs = {k: asjarray(v) for k, v in kwargs.items()}
        return fun(*args, **kwargs)

    return wrapper


def reshard(x, _spec):
    return x


class _Typeof:
    sharding = None


def typeof(_x):
    return _Typeof()
