"""The walker-batched NumPy GFMC_n step (oracle/batched.py, the CPU baseline's
implementation) against the per-walker oracle (oracle/drivers.py lrdmc_step,
jqmc_gfmc.py:4779-5166) on the same draws: the same moves, weights and
(diag, nondiag) to 1e-10 relative over several steps.  CPU only."""

import numpy as np
import pytest


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_batched_gfmc_n_matches_oracle(name):
    from jqmc_gb300 import synthetic
    from oracle import drivers as D
    from oracle.batched import BatchedGFMCn
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[name]()
    o = OracleSystem(syn.hamiltonian)
    W, steps, alat, E_scf = 3, 3, 0.2, -10.0
    r_up, r_dn = syn.initial_electrons(W, seed=21)
    r = np.concatenate([r_up, r_dn], axis=1)
    rng = np.random.default_rng(4)
    draws = [np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, 3)), rng.uniform(size=(W, 1))], axis=1)
             for _ in range(steps)]
    b = BatchedGFMCn(o, alat)
    wb = np.ones(W)
    rb = r.copy()
    states = [D.init_state(o, r_up[i], r_dn[i]) for i in range(W)]
    wo = np.ones(W)
    for d in draws:
        rb, wb, diag_b, nd_b, kb = b.step(rb, wb, d, E_scf)
        for i in range(W):
            wo[i], diag, nondiag, k = D.lrdmc_step(o, states[i], wo[i], d[i], alat, E_scf)
            assert k == kb[i]
            np.testing.assert_allclose([diag_b[i], nd_b[i]], [diag, nondiag], rtol=1e-10)
        np.testing.assert_allclose(wb, wo, rtol=1e-10)
        ro = np.stack([np.vstack([s.r_up, s.r_dn]) for s in states])
        np.testing.assert_allclose(rb, ro, rtol=0, atol=1e-12)
    eb, vb = b.energy(rb, draws[-1])
    for i in range(W):
        e, v = D.lrdmc_energy(o, states[i], draws[-1][i], alat)
        np.testing.assert_allclose([eb[i], vb[i]], [e, v], rtol=1e-10)


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_batched_vmc_matches_oracle(name):
    """oracle/batched.py BatchedVMC against oracle/drivers.py vmc_proposal /
    vmc_measure on the same draws: the same acceptances, positions, and
    e_L, w_L to 1e-10."""
    from jqmc_gb300 import synthetic
    from oracle import drivers as D
    from oracle.batched import BatchedVMC
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[name]()
    o = OracleSystem(syn.hamiltonian)
    W, K, Dt, eps = 3, 12, 0.4, 0.0
    r_up, r_dn = syn.initial_electrons(W, seed=23)
    r = np.concatenate([r_up, r_dn], axis=1)
    rng = np.random.default_rng(6)
    n, nd = o.n_up, o.n_dn
    idraw = np.stack([rng.integers(0, n + nd, (W, K)), rng.integers(0, n, (W, K)), rng.integers(0, max(nd, 1), (W, K)),
                      rng.integers(0, 3, (W, K))], axis=-1)
    fdraw = np.stack([rng.normal(size=(W, K)), rng.uniform(size=(W, K))], axis=-1)
    angles = rng.uniform(-np.pi, np.pi, (W, 3))
    b = BatchedVMC(o, Dt, eps)
    G, Ginv = b.init(r)
    states = [D.init_state(o, r_up[i], r_dn[i]) for i in range(W)]
    for k in range(K):
        acc = b.proposal(r, G, Ginv, idraw[:, k], fdraw[:, k])
        for i in range(W):
            assert D.vmc_proposal(o, states[i], idraw[i, k], fdraw[i, k], Dt, eps) == bool(acc[i])
    ro = np.stack([np.vstack([s.r_up, s.r_dn]) for s in states])
    np.testing.assert_allclose(r, ro, rtol=0, atol=1e-12)
    e, w = b.measure(r, G, Ginv, angles)
    for i in range(W):
        eo, wo = D.vmc_measure(o, states[i], angles[i], eps)
        np.testing.assert_allclose([e[i], w[i]], [eo, wo], rtol=1e-10)


@pytest.mark.parametrize("name", ["water_like", "ring12", "chain32"])
def test_shell_ao_values_match_oracle(name):
    """oracle/batched.py's shell-by-shell AO values equal oracle.ao.ao_value."""
    from jqmc_gb300 import synthetic
    from oracle.ao import ao_value
    from oracle.batched import ShellAO
    from oracle.wf import OracleSystem
    o = OracleSystem(synthetic.SYSTEMS[name]().hamiltonian)
    pts = np.random.default_rng(8).normal(scale=3.0, size=(300, 3)) + o.R.mean(axis=0)
    for tab in [o.tab_up] + ([o.tab_j3] if o.j3 is not None else []):
        ref = ao_value(tab, pts).T
        got = ShellAO(tab).values(pts)
        assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
