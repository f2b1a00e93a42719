"""An immutable, hashable mapping (the frozendict package the reference imports; part of the
JAX stand-in used to run the reference for golden vectors)."""


class frozendict(dict):  # noqa: N801
    def __hash__(self):
        return hash(tuple(sorted(self.items())))

    def _ro(self, *a, **k):
        raise TypeError('frozendict is immutable')

    __setitem__ = __delitem__ = clear = pop = popitem = setdefault = update = _ro

    def copy(self, **add):
        d = dict(self)
        d.update(add)
        return frozendict(d)
