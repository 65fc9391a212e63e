"""The oracle's closed-form d ln|psi| / d theta against central finite differences
(h = 1e-5) of the oracle's ln|psi|, which the golden fixtures pin to the
reference.  Matrix blocks are checked on a seeded sample of entries plus the
one-body column of the J3 block."""

import numpy as np
import pytest

FD_RTOL = 1e-7   # central differences at h = 1e-5: truncation ~h^2, rounding ~1e-16/h


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_oracle_adjoints_match_finite_differences(name):
    from jqmc_gb300 import synthetic
    from oracle import adjoint as AD
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[name]()
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(2, seed=31)
    rng = np.random.default_rng(5)
    A3 = o.j3_mat.shape[0]
    P, Q = o.lam_p.shape
    j3e = [(int(rng.integers(A3)), int(rng.integers(A3 + 1))) for _ in range(10)] + [(i, A3) for i in range(3)]
    le = [(int(rng.integers(P)), int(rng.integers(Q))) for _ in range(10)]
    for w in range(2):
        an = AD.dlnpsi_dparams(o, r_up[w], r_dn[w])
        fd = AD.fd_dlnpsi_dparams(o, r_up[w], r_dn[w], j3_entries=j3e, lam_entries=le)
        assert set(an) == {"j1_param", "j2_param", "j3_matrix", "lambda_matrix"}
        assert an["j3_matrix"].shape == (A3, A3 + 1)
        assert an["lambda_matrix"].shape == np.asarray(syn.hamiltonian.wavefunction_data.geminal_data.lambda_matrix).shape
        for k in an:
            a, f = np.asarray(an[k], dtype=float), np.asarray(fd[k], dtype=float)
            m = np.isfinite(f)
            scale = max(np.max(np.abs(a)), 1e-300)
            assert np.max(np.abs(a[m] - f[m])) <= FD_RTOL * scale, k
