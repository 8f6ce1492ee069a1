"""jax.tree_util for NamedTuples and plain containers."""


def tree_map(f, *trees):
    t0 = trees[0]
    if isinstance(t0, tuple) and hasattr(t0, "_fields"):
        return type(t0)(*[tree_map(f, *[getattr(t, n) for t in trees]) for n in t0._fields])
    if isinstance(t0, (list, tuple)):
        return type(t0)(tree_map(f, *xs) for xs in zip(*trees))
    if isinstance(t0, dict):
        return {k: tree_map(f, *[t[k] for t in trees]) for k in t0}
    if t0 is None:
        return None
    return f(*trees)


def register_pytree_node_class(cls):
    return cls


def register_pytree_node(*a, **k):
    return None
