"""``jax.tree`` stand-in (map over dicts/tuples/lists)."""


def map(f, tree, *rest):  # noqa: A001 - mirrors jax.tree.map
    if isinstance(tree, dict):
        return {k: map(f, tree[k], *(r[k] for r in rest)) for k in tree}
    if isinstance(tree, (tuple, list)):
        return type(tree)(map(f, t, *(r[i] for r in rest)) for i, t in enumerate(tree))
    return f(tree, *rest)
