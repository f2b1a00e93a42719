"""jax.numpy on numpy: every name resolves to numpy's (float64 stays float64); reductions
also take a list of axes, as jax.numpy's do."""
import functools as _ft

import numpy as _np

ndarray = _np.ndarray
linalg = _np.linalg


def _axis_tuple(f):
    @_ft.wraps(f)
    def g(a, axis=None, *args, **kwargs):
        if isinstance(axis, list):
            axis = tuple(axis)
        if 'axis' in kwargs and isinstance(kwargs['axis'], list):
            kwargs['axis'] = tuple(kwargs['axis'])
        return f(a, axis, *args, **kwargs)
    return g


for _n in ('mean', 'sum', 'var', 'std', 'max', 'min', 'all', 'any', 'prod', 'squeeze',
           'count_nonzero', 'nanmean', 'nansum'):
    globals()[_n] = _axis_tuple(getattr(_np, _n))


def expand_dims(a, axis):
    return _np.expand_dims(a, tuple(axis) if isinstance(axis, list) else axis)


def __getattr__(name):
    return getattr(_np, name)
