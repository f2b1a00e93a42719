"""TEST INFRASTRUCTURE: a numpy stand-in for the parts of JAX (the jax 0.4 public API) that
the reference's analytic NNGP/NTK path calls, so that the reference's own rules can run where
JAX is not installed and write golden vectors (tests/golden/make_reference_golden.py). Only that
script puts this directory on sys.path; nothing else imports it.

Each function restates the documented semantics of its JAX counterpart in numpy: arrays are
numpy arrays (float64 inputs stay float64, as under jax_enable_x64); convolutions are
cross-correlations with lax's SAME / VALID padding rule; transformations that only matter for
tracing or differentiation (jit, custom_jvp) are identities, and eval_shape runs the function on
zero arrays. Anything not provided raises StandInMissing (deliberately not a
NotImplementedError, which the reference catches in places) when used."""
import functools

import numpy as _np

from . import core, dtypes, image, interpreters, lax, nn, ops, random, scipy, tree_util  # noqa: F401
from . import numpy  # noqa: F401
from . import example_libraries  # noqa: F401
from ._missing import StandInMissing, missing_attr  # noqa: F401
from .core import ShapedArray  # noqa: F401

Array = _np.ndarray
__version__ = '0.4.30-numpy-stand-in'


class ShapeDtypeStruct:
    def __init__(self, shape, dtype):
        self.shape = tuple(shape)
        self.dtype = _np.dtype(dtype)
        self.ndim = len(self.shape)
        self.size = int(_np.prod(self.shape)) if self.shape else 1


def _concrete(x):
    if isinstance(x, (ShapeDtypeStruct, ShapedArray)):
        return _np.zeros(x.shape, x.dtype)
    return x


def eval_shape(fun, *args, **kwargs):
    """Runs fun on zero arrays of the given shapes and returns the output shapes."""
    is_leaf = lambda x: isinstance(x, (ShapeDtypeStruct, ShapedArray))
    args = tree_util.tree_map(_concrete, args, is_leaf=is_leaf)
    out = fun(*args, **kwargs)
    return tree_util.tree_map(lambda y: ShapeDtypeStruct(_np.shape(y), _np.result_type(y)), out)


def jit(fun=None, **_):
    if fun is None:
        return lambda f: f
    return fun


def vmap(fun, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = next(_np.shape(a)[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = [fun(*[a if ax is None else _np.take(a, i, axis=ax) for a, ax in zip(args, axes)])
                for i in range(n)]
        return tree_util.tree_map(lambda *ys: _np.moveaxis(_np.stack(ys), 0, out_axes), *outs)
    return mapped


class custom_jvp:  # noqa: N801
    """Forward evaluation only: the rule's own function."""

    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun
        functools.update_wrapper(self, fun)

    def defjvp(self, jvp, symbolic_zeros=False):
        self.jvp = jvp
        return jvp

    def __call__(self, *args, **kwargs):
        return self.fun(*args, **kwargs)


def default_backend():
    return 'cpu'


class _Config:
    def update(self, *_):
        pass


config = _Config()


def __getattr__(name):
    return missing_attr(name, placeholder=True)
