"""Space-warp weights of the force estimator, restated in NumPy (test infrastructure).

omega_{I i} = |r_i - R_I|^-4 / sum_J |r_i - R_J|^-4 (jqmc/swct.py:20-60) and
domega_I = sum_i grad_{r_i} omega_{I i} (jqmc/swct.py:90-110, there by automatic
differentiation; here in closed form: grad omega_I = omega_I (g_I - sum_J
omega_J g_J) with g_J = grad ln |r - R_J|^-4 = -4 (r - R_J) / |r - R_J|^2).
Pinned against the reference's _evaluate_swct_omega_debug /
_evaluate_swct_domega_debug (tests/golden).
"""

import numpy as np


def omega(R, r):
    """(M, Ne) weights for nuclei R (M, 3) and electrons r (Ne, 3)."""
    d = np.asarray(r, float)[None, :, :] - np.asarray(R, float)[:, None, :]
    k = np.sum(d * d, axis=-1) ** -2
    return k / np.sum(k, axis=0, keepdims=True)


def domega(R, r):
    """(M, 3) sum over electrons of grad_{r_i} omega_{I i}."""
    d = np.asarray(r, float)[None, :, :] - np.asarray(R, float)[:, None, :]
    d2 = np.sum(d * d, axis=-1)
    k = d2 ** -2
    w = k / np.sum(k, axis=0, keepdims=True)                 # (M, Ne)
    g = -4.0 * d / d2[..., None]                            # (M, Ne, 3)
    gbar = np.sum(w[..., None] * g, axis=0, keepdims=True)  # (1, Ne, 3)
    return np.sum(w[..., None] * (g - gbar), axis=1)
