"""Keys and samplers: values are reproducible but not JAX's bit streams (the analytic path
uses them only for parameter shapes)."""
import numpy as np


def _rng(key):
    k = np.asarray(key).astype(np.uint64).ravel()
    return np.random.default_rng([int(v) for v in k] or [0])


def PRNGKey(seed):  # noqa: N802
    return np.array([0, int(seed) & 0xffffffff], np.uint32)


def split(key, num=2):
    return _rng(key).integers(0, 2 ** 32, size=(num, 2), dtype=np.uint64).astype(np.uint32)


def fold_in(key, data):
    return _rng(np.append(np.asarray(key), int(data) & 0xffffffff)).integers(
        0, 2 ** 32, size=(2,), dtype=np.uint64).astype(np.uint32)


def normal(key, shape=(), dtype=np.float64):
    return _rng(key).standard_normal(tuple(shape)).astype(dtype)


def uniform(key, shape=(), dtype=np.float64, minval=0., maxval=1.):
    return _rng(key).uniform(minval, maxval, tuple(shape)).astype(dtype)


def bernoulli(key, p=0.5, shape=None):
    return _rng(key).random(() if shape is None else tuple(shape)) < p


def randint(key, shape, minval, maxval, dtype=np.int64):
    return _rng(key).integers(minval, maxval, tuple(shape)).astype(dtype)
