"""LRDMC forces (jqmc_gfmc.py:1810-2000, :5842-6040, :6694-6800, without space
warp): d e_L/dR of the LRDMC local energy (GPU five-point differences) against
the same differences of the oracle's LRDMC energy, and the GFMC_n / GFMC_t
drivers' force observables and get_aF."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_lrdmc_energy_gradient_matches_oracle_differences():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.forces import STENCIL, LRDMCEnergyGradientFD, displaced
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    ham = syn.hamiltonian
    r_up, r_dn = syn.initial_electrons(2, seed=61)
    rng = np.random.default_rng(62)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (2, 3)), rng.uniform(size=(2, 1))], axis=-1)
    h, alat = 5e-4, 0.2
    got = LRDMCEnergyGradientFD(ham, alat, h=h)(r_up, r_dn, torch.as_tensor(dr, device="cuda")).cpu().numpy()
    for I in range(ham.structure_data.natom):
        for k in range(3):
            o = [OracleSystem(displaced(ham, I, k, off * h)) for off, _ in STENCIL]
            for w in range(2):
                e = [D.lrdmc_energy(oo, D.init_state(oo, r_up[w], r_dn[w]), dr[w], alat)[0] for oo in o]
                fd = sum(wt * ee for ee, (_, wt) in zip(e, STENCIL)) / h
                assert abs(got[w, I, k] - fd) < 1e-6 * max(1.0, abs(fd)), (I, k, w, got[w, I, k], fd)


@pytest.mark.parametrize("driver", ["GFMC_n", "GFMC_t"])
def test_gfmc_forces(driver):
    from jqmc_gb300 import synthetic
    from jqmc_gb300 import jqmc_gfmc as G
    syn = synthetic.water_like()
    kw = dict(num_walkers=32, mcmc_seed=5, alat=0.2, num_gfmc_collect_steps=2, comput_position_deriv=True)
    if driver == "GFMC_n":
        g = G.GFMC_n(syn.hamiltonian, num_mcmc_per_measurement=5, **kw)
    else:
        g = G.GFMC_t(syn.hamiltonian, tau=0.01, **kw)
    g.run(9)
    F, Fstd = g.get_aF(num_mcmc_warmup_steps=1, num_mcmc_bin_blocks=3)
    assert F.shape == (3, 3) and np.all(np.isfinite(F)) and np.all(Fstd >= 0)
    hf, pp, elpp = g._forces.arrays(0)
    assert hf.shape == (9, 1, 3, 3) and pp.shape == hf.shape and elpp.shape == hf.shape
    assert np.all(np.isfinite(hf)) and np.all(np.isfinite(pp))
    assert not g.walkers.status.any()
