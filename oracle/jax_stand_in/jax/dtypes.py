import numpy as np


def canonicalize_dtype(dtype):
    return np.dtype(dtype)
