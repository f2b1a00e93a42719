"""Pytrees: tuples, lists, dicts, namedtuples, None (no leaves) and registered classes."""
import collections

_registry = {}


def register_pytree_node(cls, flatten, unflatten):
    _registry[cls] = (flatten, unflatten)


def _is_namedtuple(x):
    return isinstance(x, tuple) and hasattr(x, '_fields')


def _children(x):
    """(children, rebuild) for a container, or None for a leaf."""
    t = type(x)
    if t in _registry:
        flat, unflat = _registry[t]
        data, meta = flat(x)
        return list(data), lambda ch: unflat(meta, tuple(ch))
    if _is_namedtuple(x):
        return list(x), lambda ch: t(*ch)
    if isinstance(x, (tuple, list)):
        return list(x), lambda ch: t(ch)
    if isinstance(x, dict):
        keys = sorted(x.keys())
        return [x[k] for k in keys], lambda ch: t(zip(keys, ch)) if t is not dict else dict(zip(keys, ch))
    return None


def tree_map(f, tree, *rest, is_leaf=None):
    def rec(x, *ys):
        if is_leaf is not None and is_leaf(x):
            return f(x, *ys)
        if x is None:
            return None
        c = _children(x)
        if c is None:
            return f(x, *ys)
        ch, rebuild = c
        ych = []
        for y in ys:
            cy = _children(y)
            if cy is None or len(cy[0]) != len(ch):
                raise ValueError('tree_map: trees of different structure')
            ych.append(cy[0])
        return rebuild([rec(a, *[yc[i] for yc in ych]) for i, a in enumerate(ch)])
    return rec(tree, *rest)


def tree_leaves(tree, is_leaf=None):
    out = []

    def rec(x):
        if is_leaf is not None and is_leaf(x):
            out.append(x)
            return
        if x is None:
            return
        c = _children(x)
        if c is None:
            out.append(x)
            return
        for a in c[0]:
            rec(a)
    rec(tree)
    return out


def tree_all(tree):
    return all(tree_leaves(tree))


def tree_flatten(tree, is_leaf=None):
    leaves = tree_leaves(tree, is_leaf)

    def unflatten(new_leaves):
        it = iter(new_leaves)
        return tree_map(lambda _: next(it), tree, is_leaf=is_leaf)
    return leaves, unflatten


def tree_unflatten(treedef, leaves):
    return treedef(leaves)


def tree_reduce(f, tree, initializer=None):
    import functools
    leaves = tree_leaves(tree)
    return functools.reduce(f, leaves) if initializer is None else functools.reduce(f, leaves, initializer)


Partial = __import__('functools').partial
_ = collections
