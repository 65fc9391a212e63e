"""Sampled <E> of the drivers against the oracle on the same draws.

The drivers draw their own random numbers (seeded torch generators); the test
records every draw they use and replays them through the CPU oracle, walker by
walker, so both follow the same Markov chain.  Equal trajectories make the
sampled energies equal to round-off: the per-measurement local energies and
weights agree to 1e-9 relative, and get_E (the weighted jackknife of
jqmc_mcmc.py:1064-1189 / jqmc_gfmc.py:136-152) agrees to 1e-9 relative, far
inside its statistical error.  VMC: MCMC.run on water_like (Metropolis blocks
of jqmc_mcmc.py:4278-4533, E_L and w_L of :725-747).  LRDMC: GFMC_n.run on
water_like (projections of jqmc_gfmc.py:4779-5166, the energy of :5361-5640, the
comb reconfiguration of :2010-2090)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_mcmc_sampled_energy_equals_oracle():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    W, K, B = 6, 10, 24
    m = MCMC(syn.hamiltonian, mcmc_seed=11, num_walkers=W, num_mcmc_per_measurement=K, Dt=0.4, epsilon_AS=0.0)
    r0 = m.walkers.r.cpu().numpy().copy()
    used = []
    draw = m.draws

    def recording(K=None):
        d = draw(K)
        used.append(tuple(x.cpu().numpy().copy() for x in d))
        return d

    m.draws = recording
    m.run(B)
    o = OracleSystem(syn.hamiltonian)
    n = o.n_up
    e_ref = np.zeros((B, W))
    w_ref = np.zeros((B, W))
    for w in range(W):
        st = D.init_state(o, r0[w, :n], r0[w, n:])
        for b, (idraw, fdraw, angles) in enumerate(used):
            D.vmc_block(o, st, idraw[w], fdraw[w], m.Dt, m.epsilon_AS)
            e_ref[b, w], w_ref[b, w] = D.vmc_measure(o, st, angles[w], m.epsilon_AS)
    np.testing.assert_allclose(m.e_L, e_ref, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(m.w_L, w_ref, rtol=1e-9, atol=1e-12)
    from jqmc_gb300.statistics import jackknife_energy
    E, Estd, _, _ = m.get_E(num_mcmc_warmup_steps=4, num_mcmc_bin_blocks=5)
    E_ref, Estd_ref, _, _ = jackknife_energy(e_ref[4:], e_ref[4:] ** 2, w_ref[4:], 5)
    assert abs(E - E_ref) <= 1e-9 * abs(E_ref) and Estd > 0
    assert abs(E - E_ref) < 0.01 * Estd


def test_gfmc_n_sampled_energy_equals_oracle():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    W, K, B = 6, 5, 12
    g = GFMC_n(syn.hamiltonian, num_walkers=W, num_mcmc_per_measurement=K, mcmc_seed=7, alat=0.2, E_scf=-10.0,
               num_gfmc_collect_steps=2)
    r0 = g.walkers.r.cpu().numpy().copy()
    used, zetas = [], []
    draw = g.draws
    block = g.run_block

    def recording(K=None):
        d = draw(K)
        used.append(d.cpu().numpy().copy())
        return d

    def recording_block(d, zeta):
        zetas.append(zeta)
        return block(d, zeta)

    g.draws = recording
    g.run_block = recording_block
    g.run(B)
    o = OracleSystem(syn.hamiltonian)
    n = o.n_up
    states = [D.init_state(o, r0[w, :n], r0[w, n:]) for w in range(W)]
    w_avg, e_blk = [], []
    for d, zeta in zip(used, zetas):
        wts = np.ones(W)
        eL = np.zeros(W)
        vd = np.zeros(W)
        for w in range(W):
            st = states[w]
            for k in range(K):
                wts[w], _, _, _ = D.lrdmc_step(o, st, wts[w], d[w, k], g.alat, g.E_scf)
            eL[w], vd[w] = D.lrdmc_energy(o, st, d[w, -1], g.alat)
        f = wts / (vd - g.E_scf)
        w_avg.append(wts.mean())
        e_blk.append(np.sum(f * eL) / np.sum(f))
        chosen = D.branch_comb(wts, zeta)
        states = [states[c].copy() for c in chosen]
    np.testing.assert_allclose(g.bare_w_L[:, 0], w_avg, rtol=1e-9)
    np.testing.assert_allclose(np.asarray(g._e_L), e_blk, rtol=1e-9)
    E, Estd, _, _ = g.get_E(num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=4)
    assert np.isfinite(E) and np.isfinite(Estd)
    from jqmc_gb300.statistics import gfmc_G_L, jackknife_energy
    ref = np.asarray(e_blk).reshape(-1, 1)
    G = gfmc_G_L(np.asarray(w_avg).reshape(-1, 1), 2)
    E_ref, _, _, _ = jackknife_energy(ref[2:][2:], (ref[2:] ** 2)[2:], G[2:], 4)
    assert abs(E - E_ref) <= 1e-9 * abs(E_ref)
