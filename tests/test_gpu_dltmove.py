"""Determinant-locality non-local moves (non_local_move='dltmove',
jqmc_gfmc.py:4980-5017, :920-946, :5553-5600) on the GPU against the oracle:
the LRDMC energy, GFMC_n and GFMC_t trajectories (positions, weights, time
left), and the drivers.  FP64 bar 1e-10 relative."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module", params=["water_like", "ring12"])
def setup(request):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem
    from oracle.wf import OracleSystem

    syn = synthetic.SYSTEMS[request.param]()
    return syn, GpuSystem(syn.hamiltonian, non_local_move="dltmove"), GpuSystem(syn.hamiltonian), OracleSystem(syn.hamiltonian)


def _draws(W, K, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 1))], axis=-1)


def test_lrdmc_energy_dltmove(setup):
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    syn, gd, gt, o = setup
    W = 3
    r_up, r_dn = syn.initial_electrons(W, seed=21)
    dr = _draws(W, 1, 22)[:, 0]
    ed, vd = WalkerSet(gd, r_up, r_dn).lrdmc_energy(torch.as_tensor(dr, device=gd.device), 0.2)
    et, _ = WalkerSet(gt, r_up, r_dn).lrdmc_energy(torch.as_tensor(dr, device=gt.device), 0.2)
    ed, vd, et = ed.cpu().numpy(), vd.cpu().numpy(), et.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        e_ref, vd_ref = D.lrdmc_energy(o, st, dr[w], 0.2, non_local_move="dltmove")
        assert abs(ed[w] - e_ref) < RTOL * max(1.0, abs(e_ref)), (ed[w], e_ref)
        assert abs(vd[w] - vd_ref) < RTOL * max(1.0, abs(vd_ref)), (vd[w], vd_ref)
        e_t, _ = D.lrdmc_energy(o, st, dr[w], 0.2)
        assert abs(et[w] - e_t) < RTOL * max(1.0, abs(e_t))
    assert np.any(np.abs(ed - et) > 1e-8)   # the Jastrow factor of the SP part makes a difference


def test_lrdmc_projection_trajectory_dltmove(setup):
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    syn, gd, _, o = setup
    W, K = 2, (6 if syn.name == "water_like" else 3)
    r_up, r_dn = syn.initial_electrons(W, seed=23)
    ws = WalkerSet(gd, r_up, r_dn)
    dr = _draws(W, K, 24)
    wt = torch.ones(W, dtype=torch.float64, device=gd.device)
    ws.lrdmc_project(torch.as_tensor(dr, device=gd.device), 0.2, 0.0, wt)
    torch.cuda.synchronize()
    r = ws.r.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        wl = 1.0
        for k in range(K):
            wl, _, _, _ = D.lrdmc_step(o, st, wl, dr[w, k], 0.2, 0.0, non_local_move="dltmove")
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert abs(float(wt[w]) - wl) < RTOL * abs(wl)
        assert rel(ws.Ginv[w].cpu().numpy(), st.Ginv) < 1e-9
    assert not ws.status.any()


def test_lrdmc_projection_t_trajectory_dltmove(setup):
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    syn, gd, _, o = setup
    W, K = 2, 8
    tau = 0.01 if syn.name == "water_like" else 0.0015
    r_up, r_dn = syn.initial_electrons(W, seed=25)
    ws = WalkerSet(gd, r_up, r_dn)
    rng = np.random.default_rng(26)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 2))], axis=-1)
    dev = gd.device
    wt = torch.ones(W, dtype=torch.float64, device=dev)
    tl = torch.full((W,), tau, dtype=torch.float64, device=dev)
    ns = torch.zeros(W, dtype=torch.int32, device=dev)
    el = torch.full((W,), np.nan, dtype=torch.float64, device=dev)
    ws.lrdmc_project_t(torch.as_tensor(dr, device=dev), 0.2, wt, tl, ns, el)
    r = ws.r.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        wl, left, steps = 1.0, tau, 0
        for k in range(K):
            if left <= 0.0:
                break
            wl, left, _, _ = D.lrdmc_step_t(o, st, wl, left, dr[w, k], 0.2, non_local_move="dltmove")
            steps += 1
        assert int(ns[w]) == steps
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert abs(float(wt[w]) - wl) < RTOL * abs(wl)
        assert abs(float(tl[w]) - left) < 1e-12
    assert not ws.status.any()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gfmc_n_dltmove_runs(precision):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    syn = synthetic.water_like()
    g = GFMC_n(syn.hamiltonian, num_walkers=64, num_mcmc_per_measurement=10, mcmc_seed=3, alat=0.2,
               num_gfmc_collect_steps=2, non_local_move="dltmove", precision=precision)
    g.run(8)
    assert np.all(np.isfinite(g.e_L))
    assert not g.walkers.status.any()
