"""ShapedArray and an evaluation context."""
import contextlib

import numpy as np

from ._missing import missing_attr


class ShapedArray:
    def __init__(self, shape, dtype, weak_type=False):
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self.ndim = len(self.shape)
        self.size = int(np.prod(self.shape)) if self.shape else 1

    def __repr__(self):
        return f'ShapedArray({self.shape}, {self.dtype})'


@contextlib.contextmanager
def eval_context():
    yield


def __getattr__(name):
    return missing_attr('core.' + name, placeholder=True)
