"""Cartesian AOs in the walker kernels (shell kind 1) against the oracle, whose
Cartesian AOs are pinned against the reference's (tests/golden/cart.npz):
AO values/gradients/Laplacians, walker initialisation and ln psi, the VMC
local energy, a VMC sweep trajectory and an LRDMC projection trajectory on
water_like with Cartesian geminal and J3 bases (tests/cart_system.py).
FP64 bar 1e-10 relative."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def setup():
    from cart_system import water_like_cartesian

    from jqmc_gb300.engine import GpuSystem
    from oracle.wf import OracleSystem
    syn, ham = water_like_cartesian()
    return syn, GpuSystem(ham), OracleSystem(ham)


def test_cartesian_ao_vgl(setup):
    from oracle.ao import ao_vgl
    syn, gs, o = setup
    pts = np.random.default_rng(41).normal(scale=2.0, size=(129, 3))
    for basis, tab in ((0, o.tab_up), (1, o.tab_j3)):
        got = gs.ao_vgl(torch.as_tensor(pts), basis).cpu().numpy()
        ref = ao_vgl(tab, pts)
        for k in range(5):
            assert rel(got[k], ref[k]) < 1e-12, (basis, k)


def test_cartesian_walker_init_and_energy(setup):
    from jqmc_gb300.engine import WalkerSet
    from oracle.wf import rotation_matrix
    syn, gs, o = setup
    W = 3
    r_up, r_dn = syn.initial_electrons(W, seed=42)
    ws = WalkerSet(gs, r_up, r_dn)
    ld, sg, jj = [x.cpu().numpy() for x in ws.log_psi()]
    ang = np.random.default_rng(43).uniform(-2 * np.pi, 2 * np.pi, size=(W, 3))
    eL, _ = ws.vmc_measure(torch.as_tensor(ang, device=gs.device), 0.0)
    eL = eL.cpu().numpy()
    assert not ws.status.any()
    for w in range(W):
        G = o.geminal(r_up[w], r_dn[w])
        assert rel(ws.G[w].cpu().numpy(), G) < RTOL
        s_ref, ld_ref = np.linalg.slogdet(G)
        assert abs(ld[w] - ld_ref) < 1e-10 * max(1.0, abs(ld_ref)) and sg[w] == s_ref
        jref = o.jastrow_total(r_up[w], r_dn[w])
        assert abs(jj[w] - jref) < RTOL * max(1.0, abs(jref))
        ref = o.local_energy(r_up[w], r_dn[w], rotation_matrix(*ang[w]).T, np.linalg.inv(G))
        assert abs(eL[w] - ref) < RTOL * max(1.0, abs(ref)), (eL[w], ref)


def test_cartesian_vmc_and_lrdmc_trajectories(setup):
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    syn, gs, o = setup
    W, K = 2, 20
    r_up, r_dn = syn.initial_electrons(W, seed=44)
    rng = np.random.default_rng(45)
    idr = np.stack([rng.integers(0, o.n_up + o.n_dn, (W, K)), rng.integers(0, o.n_up, (W, K)),
                    rng.integers(0, o.n_dn, (W, K)), rng.integers(0, 3, (W, K))], axis=-1).astype(np.int32)
    fdr = np.stack([rng.normal(size=(W, K)), rng.uniform(size=(W, K))], axis=-1)
    ws = WalkerSet(gs, r_up, r_dn)
    acc = torch.zeros(W, dtype=torch.int32, device=gs.device)
    ws.vmc_sweep(torch.as_tensor(idr, device=gs.device), torch.as_tensor(fdr, device=gs.device), 0.4, 0.0, acc)
    torch.cuda.synchronize()
    r = ws.r.cpu().numpy()
    states = []
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        assert int(acc[w]) == D.vmc_block(o, st, idr[w], fdr[w], 0.4, 0.0)
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert rel(ws.Ginv[w].cpu().numpy(), st.Ginv) < 1e-9
        states.append(st)
    KL = 5
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, KL, 3)), rng.uniform(size=(W, KL, 1))], axis=-1)
    wt = torch.ones(W, dtype=torch.float64, device=gs.device)
    ws.lrdmc_project(torch.as_tensor(dr, device=gs.device), 0.2, 0.0, wt)
    torch.cuda.synchronize()
    r = ws.r.cpu().numpy()
    for w in range(W):
        st, wl = states[w], 1.0
        for k in range(KL):
            wl, _, _, _ = D.lrdmc_step(o, st, wl, dr[w, k], 0.2, 0.0)
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert abs(float(wt[w]) - wl) < RTOL * abs(wl)
    assert not ws.status.any()
