"""Loud failure for anything of jax this stand-in does not provide."""


class StandInMissing(RuntimeError):
    """Not a NotImplementedError on purpose: the reference catches those in places."""


class _Placeholder:
    def __init__(self, name):
        self._name = name

    def __call__(self, *a, **k):
        raise StandInMissing(self._name)

    def __getattr__(self, item):
        if item.startswith('__'):
            raise AttributeError(item)
        return _Placeholder(self._name + '.' + item)

    def __repr__(self):
        return f'<stand-in placeholder {self._name}>'


def missing_attr(name, placeholder=False):
    if placeholder:
        return _Placeholder(name)
    return StandInMissing(name)
