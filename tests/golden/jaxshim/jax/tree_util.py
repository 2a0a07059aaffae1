"""``jax.tree_util`` stand-in."""


def register_dataclass(cls=None, **_kwargs):
    """Marks a dataclass as a pytree: its fields are data leaves except those whose metadata says
    ``static`` (recorded for ``lax.scan``, which slices the data leaves)."""
    if cls is None:
        return lambda c: register_dataclass(c)
    import dataclasses
    cls._shim_static = tuple(f.name for f in dataclasses.fields(cls) if f.metadata.get('static'))
    cls._shim_data = tuple(f.name for f in dataclasses.fields(cls)
                           if not f.metadata.get('static'))
    return cls
