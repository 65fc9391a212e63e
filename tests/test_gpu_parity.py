"""GPU parity: every C-ABI entry point against the CPU oracle on the same inputs.

FP64 bar: 1e-10 relative for values, ratios and energies (relative to the
largest magnitude of the compared array); accept/reject decisions and chosen
moves must coincide exactly given the same draws.
"""

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
    gs = GpuSystem(syn.hamiltonian)
    o = OracleSystem(syn.hamiltonian)
    return syn, gs, o


def test_ao_vgl(setup):
    from oracle.ao import ao_vgl
    syn, gs, o = setup
    pts = np.random.default_rng(1).normal(scale=2.0, size=(257, 3))
    got = gs.ao_vgl(torch.as_tensor(pts), 0).cpu().numpy()
    ref = ao_vgl(o.tab_up if o.mo_up is None else o.tab_up, pts)
    for k in range(5):
        assert rel(got[k], ref[k]) < 1e-12, f"det basis component {k}"
    got3 = gs.ao_vgl(torch.as_tensor(pts), 1).cpu().numpy()
    ref3 = ao_vgl(o.tab_j3, pts)
    for k in range(5):
        assert rel(got3[k], ref3[k]) < 1e-12, f"J3 basis component {k}"


def _walkers(syn, gs, W, seed):
    from jqmc_gb300.engine import WalkerSet
    r_up, r_dn = syn.initial_electrons(W, seed=seed)
    ws = WalkerSet(gs, r_up, r_dn)
    torch.cuda.synchronize()
    return ws, r_up, r_dn


def test_walker_init_and_log_psi(setup):
    syn, gs, o = setup
    ws, r_up, r_dn = _walkers(syn, gs, 3, 5)
    G = ws.G.cpu().numpy()
    Gi = ws.Ginv.cpu().numpy()
    ld, sg, jj = [x.cpu().numpy() for x in ws.log_psi()]
    assert not ws.status.any()
    for w in range(3):
        Gr = o.geminal(r_up[w], r_dn[w])
        assert rel(G[w], Gr) < RTOL
        assert rel(Gi[w], np.linalg.inv(Gr)) < 1e-9
        s_ref, ld_ref = np.linalg.slogdet(Gr)
        assert abs(ld[w] - ld_ref) < 1e-10 * max(1.0, abs(ld_ref)) and sg[w] == s_ref
        jref = o.jastrow_total(r_up[w], r_dn[w])
        assert abs(jj[w] - jref) < RTOL * max(1.0, abs(jref))
        if o.j3 is not None:
            h = o.j3_fields(r_up[w], r_dn[w])
            assert rel(ws.h3[w].cpu().numpy().T, h) < RTOL


def test_vmc_measure(setup):
    from oracle.wf import rotation_matrix
    syn, gs, o = setup
    W = 3
    ws, r_up, r_dn = _walkers(syn, gs, W, 6)
    ang = np.random.default_rng(2).uniform(-2 * np.pi, 2 * np.pi, size=(W, 3))
    eL, wL = ws.vmc_measure(torch.as_tensor(ang, device=gs.device), 0.0)
    eL = eL.cpu().numpy()
    for w in range(W):
        G = o.geminal(r_up[w], r_dn[w])
        ref = o.local_energy(r_up[w], r_dn[w], rotation_matrix(*ang[w]).T, np.linalg.inv(G))
        assert abs(eL[w] - ref) < RTOL * max(1.0, abs(ref)), (eL[w], ref)
    assert np.allclose(wL.cpu().numpy(), 1.0)


def _vmc_draws(o, W, K, seed):
    rng = np.random.default_rng(seed)
    idr = np.stack([rng.integers(0, o.n_up + o.n_dn, (W, K)), rng.integers(0, o.n_up, (W, K)),
                    rng.integers(0, o.n_dn, (W, K)), rng.integers(0, 3, (W, K))], axis=-1).astype(np.int32)
    fdr = np.stack([rng.normal(size=(W, K)), rng.uniform(size=(W, K))], axis=-1)
    return idr, fdr


def test_vmc_sweep_trajectory(setup):
    from oracle import drivers as D
    syn, gs, o = setup
    W, K = 2, 30 if syn.name == "water_like" else 12
    ws, r_up, r_dn = _walkers(syn, gs, W, 7)
    idr, fdr = _vmc_draws(o, W, K, 3)
    acc = torch.zeros(W, dtype=torch.int32, device=gs.device)
    ws.vmc_sweep(torch.as_tensor(idr, device=gs.device), torch.as_tensor(fdr, device=gs.device), 0.4, 0.0, acc)
    torch.cuda.synchronize()
    r = ws.r.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        nacc = D.vmc_block(o, st, idr[w], fdr[w], 0.4, 0.0)
        assert int(acc[w]) == nacc
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert rel(ws.Ginv[w].cpu().numpy(), st.Ginv) < 1e-9
        assert rel(ws.G[w].cpu().numpy(), st.G) < 1e-10


def _lrdmc_draws(W, K, seed):
    rng = np.random.default_rng(seed)
    return np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 1))], axis=-1)


def test_lrdmc_energy(setup):
    from oracle import drivers as D
    syn, gs, o = setup
    W = 2
    ws, r_up, r_dn = _walkers(syn, gs, W, 8)
    dr = _lrdmc_draws(W, 1, 4)[:, 0]
    eL, vd = ws.lrdmc_energy(torch.as_tensor(dr, device=gs.device), 0.2)
    eL, vd = eL.cpu().numpy(), vd.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        e_ref, vd_ref = D.lrdmc_energy(o, st, dr[w], 0.2)
        assert abs(eL[w] - e_ref) < RTOL * max(1.0, abs(e_ref)), (eL[w], e_ref)
        assert abs(vd[w] - vd_ref) < RTOL * max(1.0, abs(vd_ref)), (vd[w], vd_ref)


def test_lrdmc_projection_trajectory(setup):
    from oracle import drivers as D
    syn, gs, o = setup
    W, K = 2, (6 if syn.name == "water_like" else 3)
    ws, r_up, r_dn = _walkers(syn, gs, W, 9)
    dr = _lrdmc_draws(W, K, 5)
    wt = torch.ones(W, dtype=torch.float64, device=gs.device)
    ws.lrdmc_project(torch.as_tensor(dr, device=gs.device), 0.2, 0.0, wt)
    torch.cuda.synchronize()
    r = ws.r.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        wl = 1.0
        for k in range(K):
            wl, _, _, _ = D.lrdmc_step(o, st, wl, dr[w, k], 0.2, 0.0)
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert abs(float(wt[w]) - wl) < RTOL * abs(wl)
        assert rel(ws.Ginv[w].cpu().numpy(), st.Ginv) < 1e-9
    assert not ws.status.any()


def test_branch_and_gather(setup):
    from jqmc_gb300.engine import WalkerSet, branch_comb
    from oracle import drivers as D
    syn, gs, o = setup
    W = 64
    ws, _, _ = _walkers(syn, gs, W, 10)
    w = np.random.default_rng(11).uniform(0.2, 2.0, size=W)
    chosen = branch_comb(torch.as_tensor(w, device=gs.device), 0.37)
    ref = D.branch_comb(w, 0.37)
    assert np.array_equal(chosen.cpu().numpy(), ref)
    dst = WalkerSet.empty_like(ws)
    dst.gather_from(ws, chosen)
    assert torch.equal(dst.r, ws.r[chosen.long()])
    assert torch.equal(dst.Tup, ws.Tup[chosen.long()])


def test_lu_rebuild_refine(setup):
    """After a projection block the FP64 rebuild reproduces a fresh build from the
    positions (G, G^-1, T tables, J3 field), leaves the exact per-electron caches
    untouched, and its inverse matches the oracle's."""
    from jqmc_gb300.engine import WalkerSet
    from oracle import drivers as D
    syn, gs, o = setup
    W, K = 8, 6
    ws, _, _ = _walkers(syn, gs, W, 12)
    dr = torch.as_tensor(_lrdmc_draws(W, K + 1, 13), device=gs.device)
    wt = torch.ones(W, dtype=torch.float64, device=gs.device)
    ws.lrdmc_project(dr[:, :K].contiguous(), 0.2, 0.0, wt)
    ec, dp, dp3 = ws.ecache.clone(), ws.dphi.clone(), ws.dphi3.clone()
    ws.rebuild()
    torch.cuda.synchronize()
    assert torch.equal(ws.ecache, ec) and torch.equal(ws.dphi, dp) and torch.equal(ws.dphi3, dp3)
    r = ws.r.cpu().numpy()
    n = gs.n_up
    fresh = WalkerSet(gs, r[:, :n], r[:, n:])
    for name in ("G", "Ginv", "Tup", "Tdn", "h3"):
        assert rel(getattr(ws, name).cpu().numpy(), getattr(fresh, name).cpu().numpy()) < 1e-10, name
    last = dr[:, K].contiguous()
    e1, v1 = ws.lrdmc_energy(last, 0.2)
    e2, v2 = fresh.lrdmc_energy(last, 0.2)
    assert rel(e1.cpu().numpy(), e2.cpu().numpy()) < 1e-10
    assert rel(v1.cpu().numpy(), v2.cpu().numpy()) < 1e-10
    for w in range(2):
        st = D.init_state(o, r[w, :n], r[w, n:])
        assert rel(ws.Ginv[w].cpu().numpy(), st.Ginv) < 1e-10
    assert not ws.status.any()


def test_lrdmc_projection_t_trajectory(setup):
    """GFMC_t: projections until the time is spent, the draws split over two
    calls (the second resumes with the time left); positions, weights, time
    left, step counts and the final-step e_L against the oracle."""
    from oracle import drivers as D
    syn, gs, o = setup
    W = 3
    tau = 0.01 if syn.name == "water_like" else 0.0015
    K1, K2 = 3, 9
    ws, r_up, r_dn = _walkers(syn, gs, W, 14)
    rng = np.random.default_rng(15)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K1 + K2, 3)), rng.uniform(size=(W, K1 + K2, 2))], axis=-1)
    dev = gs.device
    wt = torch.ones(W, dtype=torch.float64, device=dev)
    tl = torch.full((W,), tau, dtype=torch.float64, device=dev)
    ns = torch.zeros(W, dtype=torch.int32, device=dev)
    el = torch.full((W,), np.nan, dtype=torch.float64, device=dev)
    total = np.zeros(W, dtype=np.int64)
    for a, b in ((0, K1), (K1, K1 + K2)):
        ws.lrdmc_project_t(torch.as_tensor(dr[:, a:b].copy(), device=dev), 0.2, wt, tl, ns, el)
        total += ns.cpu().numpy()
    r = ws.r.cpu().numpy()
    for w in range(W):
        st = D.init_state(o, r_up[w], r_dn[w])
        wl, left, steps, e_last = 1.0, tau, 0, np.nan
        for k in range(K1 + K2):
            if left <= 0.0:
                break
            wl, left, e, moved = D.lrdmc_step_t(o, st, wl, left, dr[w, k], 0.2)
            steps += 1
            if left <= 0.0:
                e_last = e
        assert total[w] == steps
        assert rel(r[w], np.vstack([st.r_up, st.r_dn])) < 1e-12
        assert abs(float(wt[w]) - wl) < RTOL * abs(wl)
        assert abs(float(tl[w]) - left) < 1e-12
        if left <= 0.0:
            assert abs(float(el[w]) - e_last) < RTOL * max(1.0, abs(e_last))
    assert not ws.status.any()
