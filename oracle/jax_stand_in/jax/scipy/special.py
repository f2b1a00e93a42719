"""jax.scipy.special on scipy."""
from scipy.special import erf, erfc, ndtr  # noqa: F401
