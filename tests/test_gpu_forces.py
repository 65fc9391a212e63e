"""Nuclear-force terms: d ln psi / dR from the adjoint kernel against central
differences of the oracle's ln|psi| with displaced nuclei, dE_L/dR (GPU central
differences) against the same differences of the oracle's local energy, and the
MCMC driver's force and parameter-derivative observables."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", ["water_like", "ring12"])
def test_dlnpsi_dR_matches_oracle_differences(name):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from jqmc_gb300.forces import displaced, dlnpsi_dR
    from oracle import adjoint as AD
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[name]()
    ham = syn.hamiltonian
    r_up, r_dn = syn.initial_electrons(2, seed=51)
    gs = GpuSystem(ham)
    got = dlnpsi_dR(WalkerSet(gs, r_up, r_dn)).cpu().numpy()
    from jqmc_gb300.forces import STENCIL
    h = 1e-5   # five-point stencil: truncation ~h^4 even where ln psi is steep
    M = ham.structure_data.natom
    atoms = range(M) if M <= 3 else (0, 5, 7)
    for I in atoms:
        for k in range(3):
            osys = [OracleSystem(displaced(ham, I, k, o * h)) for o, _ in STENCIL]
            for w in range(2):
                fd = sum(wt * AD.ln_psi(oo, r_up[w], r_dn[w]) for oo, (_, wt) in zip(osys, STENCIL)) / h
                scale = max(np.max(np.abs(got[w])), 1.0)
                assert abs(got[w, I, k] - fd) < 1e-7 * scale, (I, k, w, got[w, I, k], fd)


def test_el_gradient_matches_oracle_differences():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.forces import ELGradientFD, displaced
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    ham = syn.hamiltonian
    r_up, r_dn = syn.initial_electrons(2, seed=52)
    rng = np.random.default_rng(8)
    ang = rng.uniform(-2 * np.pi, 2 * np.pi, (2, 3))
    from jqmc_gb300.forces import STENCIL
    h = 5e-4
    g = ELGradientFD(ham, h=h)
    got = g(r_up, r_dn, torch.as_tensor(ang, device="cuda")).cpu().numpy()
    for I in range(ham.structure_data.natom):
        for k in range(3):
            o = [OracleSystem(displaced(ham, I, k, off * h)) for off, _ in STENCIL]
            for w in range(2):
                e = [D.vmc_measure(oo, D.init_state(oo, r_up[w], r_dn[w]), ang[w], 0.0)[0] for oo in o]
                fd = sum(wt * ee for ee, (_, wt) in zip(e, STENCIL)) / h
                assert abs(got[w, I, k] - fd) < 1e-6 * max(1.0, abs(fd)), (I, k, w, got[w, I, k], fd)


def test_mcmc_forces_and_parameter_derivatives():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    syn = synthetic.water_like()
    m = MCMC(syn.hamiltonian, mcmc_seed=2, num_walkers=32, num_mcmc_per_measurement=10, Dt=0.4, epsilon_AS=0.0,
             comput_log_WF_param_deriv=True, comput_position_deriv=True, use_swct=False)
    m.run(12)
    F, Fstd = m.get_aF(num_mcmc_warmup_steps=2, num_mcmc_bin_blocks=5)
    assert F.shape == (3, 3) and np.all(np.isfinite(F)) and np.all(Fstd > 0)
    d = m.dln_Psi_dc
    assert d["j3_matrix"].shape == (12, 32, 20, 21)
    assert d["lambda_matrix"].shape[:2] == (12, 32)


def _warp(o_R, r, I, k, delta):
    from oracle import swct
    om = swct.omega(o_R, r)
    out = r.copy()
    out[:, k] += delta * om[I]
    return out


def test_space_warp_terms_match_oracle_differences():
    """force_HF with the electrons warped along each displaced nucleus, and
    sum_i omega d ln psi/dr_i, against the same differences of the oracle."""
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem
    from jqmc_gb300.forces import STENCIL, ELGradientFD, displaced, warped_dlnpsi
    from oracle import adjoint as AD
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    ham = syn.hamiltonian
    n = syn.n_up
    r_up, r_dn = syn.initial_electrons(2, seed=53)
    ang = np.random.default_rng(9).uniform(-2 * np.pi, 2 * np.pi, (2, 3))
    h = 5e-4
    got = ELGradientFD(ham, h=h, warp=True)(r_up, r_dn, torch.as_tensor(ang, device="cuda")).cpu().numpy()
    gl = warped_dlnpsi(GpuSystem(ham), r_up, r_dn, h=h).cpu().numpy()
    R = ham.structure_data.positions
    o0 = OracleSystem(ham)
    for I in range(ham.structure_data.natom):
        for k in range(3):
            osys = [OracleSystem(displaced(ham, I, k, off * h)) for off, _ in STENCIL]
            for w in range(2):
                r = np.vstack([r_up[w], r_dn[w]])
                e, l = [], []
                for oo, (off, _) in zip(osys, STENCIL):
                    rw = _warp(R, r, I, k, off * h)
                    e.append(D.vmc_measure(oo, D.init_state(oo, rw[:n], rw[n:]), ang[w], 0.0)[0])
                    l.append(AD.ln_psi(o0, rw[:n], rw[n:]))
                fd_e = sum(wt * x for x, (_, wt) in zip(e, STENCIL)) / h
                fd_l = sum(wt * x for x, (_, wt) in zip(l, STENCIL)) / h
                assert abs(got[w, I, k] - fd_e) < 1e-6 * max(1.0, abs(fd_e)), (I, k, w, got[w, I, k], fd_e)
                assert abs(gl[w, I, k] - fd_l) < 1e-6 * max(1.0, abs(fd_l)), (I, k, w, gl[w, I, k], fd_l)


def test_mcmc_space_warp_forces():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    syn = synthetic.water_like()
    m = MCMC(syn.hamiltonian, mcmc_seed=4, num_walkers=16, num_mcmc_per_measurement=10, Dt=0.4, epsilon_AS=0.0,
             comput_position_deriv=True)   # use_swct defaults to True, as in the reference
    m.run(6)
    F, Fstd = m.get_aF(num_mcmc_warmup_steps=1, num_mcmc_bin_blocks=5)
    assert F.shape == (3, 3) and np.all(np.isfinite(F)) and np.all(Fstd > 0)
