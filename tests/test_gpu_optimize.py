"""SR wavefunction optimisation through the MCMC driver on the GPU
(jqmc_mcmc.py:1372-1700, :2368-3800): derivative samples from the walker
kernels, generalized forces, the SR solve on the device against the same solve
on the host, and run_optimize steps that move the parameters, keep the J3
symmetry and reset the sampler."""

import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_sr_optimisation_on_the_gpu():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    from jqmc_gb300.variational import get_variational_blocks, sr_direction
    syn = synthetic.water_like()
    wf0 = syn.hamiltonian.wavefunction_data
    m = MCMC(syn.hamiltonian, mcmc_seed=4, num_walkers=128, num_mcmc_per_measurement=10, Dt=0.4, epsilon_AS=0.0,
             comput_log_WF_param_deriv=True)
    m.run(12)
    blocks = get_variational_blocks(wf0)
    K = sum(b.size for b in blocks)
    O = m.get_dln_WF(blocks, num_mcmc_warmup_steps=2)
    assert O.shape == (10, 128, K) and np.all(np.isfinite(O))
    f, f_std = m.get_gF(num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=5, blocks=blocks)
    assert f.shape == (K,) and np.all(np.isfinite(f)) and np.all(f_std >= 0)
    on_gpu = sr_direction(O, m.e_L[2:], m.w_L[2:], 1e-3, cg_flag=False, device=m.sys.device)
    on_cpu = sr_direction(O, m.e_L[2:], m.w_L[2:], 1e-3, cg_flag=False, device="cpu")
    scale = np.max(np.abs(on_cpu.theta))
    np.testing.assert_allclose(on_gpu.theta, on_cpu.theta, rtol=1e-6, atol=1e-8 * scale)
    np.testing.assert_allclose(on_gpu.f, on_cpu.f, rtol=1e-10, atol=1e-12 * np.max(np.abs(on_cpu.f)))
    # CG to |r| <= 1e-9 on the normalised system (eigenvalues >= epsilon): |d theta_n| <= 1e-6
    cg = sr_direction(O, m.e_L[2:], m.w_L[2:], 1e-3, cg_flag=True, cg_tol=1e-9, cg_max_iter=5000,
                      device=m.sys.device)
    d = np.sqrt(on_cpu.diag_S)
    np.testing.assert_allclose(cg.theta * d, on_cpu.theta * d, rtol=0, atol=1e-5)

    # a small delta keeps J1 and J2 (both 1.0) well away from zero on 1280 noisy samples
    hist = m.run_optimize(num_mcmc_steps=12, num_opt_steps=2, num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=5,
                          optimizer_kwargs=dict(delta=2e-4, cg_max_iter=5000))
    assert len(hist) == 2 and all(np.isfinite(h["E"]) and h["E_std"] > 0 for h in hist)
    assert m.mcmc_counter == 0
    wf1 = m.hamiltonian_data.wavefunction_data
    b0 = wf0.jastrow_data.jastrow_two_body_data.jastrow_2b_param
    b1 = wf1.jastrow_data.jastrow_two_body_data.jastrow_2b_param
    assert b1 != b0
    jm = wf1.jastrow_data.jastrow_three_body_data.j_matrix
    np.testing.assert_array_equal(jm[:, :-1], jm[:, :-1].T)
    assert not np.array_equal(jm, wf0.jastrow_data.jastrow_three_body_data.j_matrix)
    m.run(3)
    assert m.e_L.shape == (3, 128) and np.all(np.isfinite(m.e_L))
    assert not m.walkers.status.any()
