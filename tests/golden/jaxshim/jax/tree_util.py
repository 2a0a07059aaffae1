"""``jax.tree_util`` stand-in."""


def register_dataclass(cls=None, **_kwargs):
    if cls is None:
        return lambda c: c
    return cls
