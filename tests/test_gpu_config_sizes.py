"""The walker kernels at the benchmark configurations' own sizes, checked
against the oracle on the same draws.

* chain32 (config 2's system, 96 electrons, 736 AOs, ECP): FP64 GFMC_n
  trajectories of three walkers against the walker-batched NumPy step
  (oracle/batched.py, itself pinned to oracle/drivers.py lrdmc_step by
  test_oracle_batched.py): the same moves, weights to 1e-10.
* config 1 (LRDMC ring12, 8192 walkers): the whole batch projected on the GPU,
  four walkers spread over the batch replayed on the CPU.
* config 0 (VMC water-like, 1024 walkers, blocks of 40 proposals with E_L per
  block): the MCMC driver's recorded draws replayed for three walkers through
  oracle/drivers.py (jqmc_mcmc.py:4278-4533, E_L of :725-747).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _lrdmc_draws(W, K, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 1))], axis=-1)


def _replay_batched(o, r0, dr, alat, E_scf):
    from oracle.batched import BatchedGFMCn
    b = BatchedGFMCn(o, alat)
    r = r0.copy()
    w = np.ones(r.shape[0])
    for k in range(dr.shape[1]):
        r, w, _, _, _ = b.step(r, w, dr[:, k], E_scf)
    return r, w


def test_chain32_fp64_lrdmc_trajectory():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from oracle.wf import OracleSystem
    syn = synthetic.chain32()
    gs = GpuSystem(syn.hamiltonian)
    o = OracleSystem(syn.hamiltonian)
    W, K, alat = 3, 4, 0.2
    r_up, r_dn = syn.initial_electrons(W, seed=31)
    ws = WalkerSet(gs, r_up, r_dn)
    dr = _lrdmc_draws(W, K, 32)
    wt = torch.ones(W, dtype=torch.float64, device=gs.device)
    ws.lrdmc_project(torch.as_tensor(dr, device=gs.device), alat, 0.0, wt)
    torch.cuda.synchronize()
    r_ref, w_ref = _replay_batched(o, np.concatenate([r_up, r_dn], axis=1), dr, alat, 0.0)
    np.testing.assert_allclose(ws.r.cpu().numpy(), r_ref, rtol=0, atol=1e-12)
    np.testing.assert_allclose(wt.cpu().numpy(), w_ref, rtol=1e-10)
    assert not ws.status.any()


def test_config1_ring12_8192_walkers():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from oracle.wf import OracleSystem
    syn = synthetic.ring12()
    gs = GpuSystem(syn.hamiltonian)
    o = OracleSystem(syn.hamiltonian)
    W, K, alat, E_scf = 8192, 4, 0.2, -10.0
    r_up, r_dn = syn.initial_electrons(W, seed=41)
    ws = WalkerSet(gs, r_up, r_dn)
    dr = _lrdmc_draws(W, K, 42)
    wt = torch.ones(W, dtype=torch.float64, device=gs.device)
    ws.lrdmc_project(torch.as_tensor(dr, device=gs.device), alat, E_scf, wt)
    torch.cuda.synchronize()
    assert not ws.status.any()
    w_all = wt.cpu().numpy()
    assert np.all(np.isfinite(w_all))
    pick = np.array([0, 2047, 5003, 8191])
    r0 = np.concatenate([r_up, r_dn], axis=1)[pick]
    r_ref, w_ref = _replay_batched(o, r0, dr[pick], alat, E_scf)
    np.testing.assert_allclose(ws.r[pick].cpu().numpy(), r_ref, rtol=0, atol=1e-12)
    np.testing.assert_allclose(w_all[pick], w_ref, rtol=1e-10)


def test_config0_water_vmc_1024_walkers():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    W, K, B = 1024, 40, 3
    m = MCMC(syn.hamiltonian, mcmc_seed=51, num_walkers=W, num_mcmc_per_measurement=K, Dt=0.4, epsilon_AS=0.0)
    r0 = m.walkers.r.cpu().numpy().copy()
    used = []
    draw = m.draws

    def recording(K=None):
        d = draw(K)
        used.append(tuple(x.cpu().numpy().copy() for x in d))
        return d

    m.draws = recording
    m.run(B)
    assert np.all(np.isfinite(m.e_L))
    o = OracleSystem(syn.hamiltonian)
    n = o.n_up
    for w in (0, 511, 1023):
        st = D.init_state(o, r0[w, :n], r0[w, n:])
        for b, (idraw, fdraw, angles) in enumerate(used):
            D.vmc_block(o, st, idraw[w], fdraw[w], m.Dt, m.epsilon_AS)
            e, wl = D.vmc_measure(o, st, angles[w], m.epsilon_AS)
            assert abs(m.e_L[b, w] - e) <= 1e-9 * max(1.0, abs(e)), (w, b)
            assert abs(m.w_L[b, w] - wl) <= 1e-9 * max(1.0, abs(wl)), (w, b)
