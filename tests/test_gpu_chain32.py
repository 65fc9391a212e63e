"""The 32-nucleus chain (96 electrons, 736 AOs): FP64 local energy against the
oracle, and the mixed form (displacement caches in global memory at this size)
against the FP64 form on sampled configurations."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chain():
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem
    syn = synthetic.chain32()
    return syn, GpuSystem(syn.hamiltonian)


def test_chain32_fp64_energy_matches_oracle(chain):
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn, gs = chain
    r_up, r_dn = syn.initial_electrons(1, seed=3)
    ws = WalkerSet(gs, r_up, r_dn, precision="fp64")
    dr = np.array([[0.3, -1.1, 2.0, 0.5]])
    eL, vd = ws.lrdmc_energy(torch.as_tensor(dr, device=gs.device), 0.2)
    o = OracleSystem(syn.hamiltonian)
    st = D.init_state(o, r_up[0], r_dn[0])
    e_ref, vd_ref = D.lrdmc_energy(o, st, dr[0], 0.2)
    assert abs(float(eL[0]) - e_ref) < 1e-10 * max(1.0, abs(e_ref)), (float(eL[0]), e_ref)
    assert abs(float(vd[0]) - vd_ref) < 1e-10 * max(1.0, abs(vd_ref))


def test_chain32_mixed_vs_fp64(chain):
    from jqmc_gb300.engine import WalkerSet
    syn, gs = chain
    W = 128
    r_up, r_dn = syn.initial_electrons(W, seed=4)
    eq = WalkerSet(gs, r_up, r_dn, precision="fp64")
    rng = np.random.default_rng(2)
    K = 40
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 1))], axis=-1)
    w = torch.ones(W, dtype=torch.float64, device=gs.device)
    eq.lrdmc_project(torch.as_tensor(dr, device=gs.device), 0.2, 0.0, w)
    r = eq.r.cpu().numpy()
    n = gs.n_up
    a = WalkerSet(gs, r[:, :n], r[:, n:], precision="fp64")
    b = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed")
    assert b.dcache is not None
    d1 = torch.as_tensor(dr[:, -1], device=gs.device)
    e64, _ = a.lrdmc_energy(d1, 0.2)
    e32, _ = b.lrdmc_energy(d1, 0.2)
    de = (e32 - e64).cpu().numpy()
    rms = float(np.sqrt(np.mean(de**2)))
    print(f"chain32: mixed vs fp64 e_L rms {rms:.3e} Ha, mean {np.mean(de):.2e}")
    assert rms <= 1e-5
    assert not a.status.any() and not b.status.any()
