"""The reference-shaped drivers (MCMC, GFMC_n) run end to end on the GPU."""

import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_mcmc_runs_and_reports_energy():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    syn = synthetic.water_like()
    m = MCMC(syn.hamiltonian, mcmc_seed=1, num_walkers=64, num_mcmc_per_measurement=20, Dt=0.4, epsilon_AS=0.0)
    m.run(30)
    assert m.e_L.shape == (30, 64) and np.all(np.isfinite(m.e_L))
    E, Estd, V, Vstd = m.get_E(num_mcmc_warmup_steps=10, num_mcmc_bin_blocks=5)
    assert np.isfinite(E) and Estd > 0
    acc = m.accepted_moves / (m.accepted_moves + m.rejected_moves)
    assert 0.05 < acc < 0.99
    assert not m.walkers.status.any()


def test_gfmc_n_runs_and_reports_energy():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    syn = synthetic.water_like()
    g = GFMC_n(syn.hamiltonian, num_walkers=64, num_mcmc_per_measurement=10, mcmc_seed=3, alat=0.2, num_gfmc_collect_steps=2)
    g.run(14)
    assert np.all(np.isfinite(g.e_L))
    E, Estd, _, _ = g.get_E(num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=5)
    assert np.isfinite(E)
    assert not g.walkers.status.any()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gfmc_t_runs_and_reports_energy(precision):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_t
    syn = synthetic.water_like()
    g = GFMC_t(syn.hamiltonian, num_walkers=64, mcmc_seed=5, tau=0.05, alat=0.2, num_gfmc_collect_steps=2,
               precision=precision, draws_per_call=16)
    g.run(12)
    assert np.all(np.isfinite(g.e_L)) and g.e_L.shape == (10, 1)
    assert np.all(g.average_projection_counter > 1.0)
    E, Estd, _, _ = g.get_E(num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=4)
    assert np.isfinite(E)
    assert not g.walkers.status.any()
