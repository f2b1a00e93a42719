"""jax.nn: the activations the analytic path names."""
import numpy as np
from scipy.special import erf as _erf


def relu(x):
    return np.maximum(x, 0)


def gelu(x, approximate=True):
    if approximate:
        return 0.5 * x * (1 + np.tanh(np.sqrt(2 / np.pi) * (x + 0.044715 * x ** 3)))
    return 0.5 * x * (1 + _erf(x / np.sqrt(2)))


def softmax(x, axis=-1):
    e = np.exp(x - np.max(x, axis=axis, keepdims=True))
    return e / np.sum(e, axis=axis, keepdims=True)
