"""jax.scipy.linalg on scipy.linalg (the same factor / solve conventions)."""
from scipy.linalg import cho_factor, cho_solve, eigh, solve_triangular  # noqa: F401
