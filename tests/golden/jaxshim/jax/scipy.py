"""jax.scipy -> SciPy."""
import scipy.linalg as linalg  # noqa: F401
import scipy.special as special  # noqa: F401
