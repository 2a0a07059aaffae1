"""``jax.debug`` stand-in: prints eagerly."""


def print(fmt, *args, **kwargs):  # noqa: A001 - mirrors jax.debug.print
    __builtins__['print'](fmt.format(*args, **kwargs)) if isinstance(__builtins__, dict) \
        else __builtins__.print(fmt.format(*args, **kwargs))
