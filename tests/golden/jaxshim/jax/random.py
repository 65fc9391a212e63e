"""jax.random is not reproducible with NumPy; calls raise."""


def _raise(*a, **k):
    raise NotImplementedError("jax.random is not available in the NumPy stand-in")


PRNGKey = split = normal = uniform = randint = fold_in = _raise
