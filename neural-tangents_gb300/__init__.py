"""nt_gb300: the analytic NNGP/NTK path of neural-tangents on GB300 (sm_103a).

Drop-in for ``neural_tangents.stax`` kernel functions, ``neural_tangents.batch``
and ``neural_tangents.predict.gradient_descent_mse``; every kernel runs in the
hand-written CUDA library libntgb300.so behind include/nt_gb300.h.
"""
from . import stax  # noqa: F401
from . import predict  # noqa: F401
from . import tune  # noqa: F401
from .batching import batch, CapturedBatch  # noqa: F401
from .kernel import Kernel  # noqa: F401

__version__ = '0.1.0'
