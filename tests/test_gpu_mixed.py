"""Mixed-precision form (FP32 tables, AO values, ratios and rank-1 updates;
FP64 gradients/Laplacians, energies, weights and rebuilds) against the plain
FP64 form on the same configurations and the same draws.

Configurations are equilibrated first (60 FP64 projections from the initial
electron placement), as the workload compares sampled configurations.
Bars: per-configuration |dE_L| <= 1e-5 Ha rms (the workload's bar), its mean
(the bias that would reach <E>) below 1e-5 Ha; over K projections with the same
draws at least 95 % of walkers take the same moves and their weights agree to
5e-6 relative per projection (the weight is a product of K factors).
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["water_like", "ring12"])
def pair(request):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    syn = synthetic.SYSTEMS[request.param]()
    gs = GpuSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(256, seed=21)
    eq = WalkerSet(gs, r_up, r_dn, precision="fp64")
    rng = np.random.default_rng(1)
    K = 60
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (256, K, 3)), rng.uniform(size=(256, K, 1))], axis=-1)
    w = torch.ones(256, dtype=torch.float64, device=gs.device)
    eq.lrdmc_project(torch.as_tensor(dr, device=gs.device), 0.2, 0.0, w)
    r = eq.r.cpu().numpy()
    n = gs.n_up
    w64 = WalkerSet(gs, r[:, :n], r[:, n:], precision="fp64")
    w32 = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed")
    torch.cuda.synchronize()
    return syn, gs, w64, w32


def test_mixed_rebuild_matches_fp64(pair):
    syn, gs, w64, w32 = pair
    gi64 = w64.Ginv
    gi32 = w32.Ginv.double()
    rel = ((gi32 - gi64).abs().amax(dim=(1, 2)) / gi64.abs().amax(dim=(1, 2)))
    assert float(rel.max()) < 1e-5
    t = (w32.Tup.double() - w64.Tup).abs().amax(dim=(1, 2)) / w64.Tup.abs().amax(dim=(1, 2))
    assert float(t.max()) < 1e-5
    assert not w32.status.any()


def test_mixed_local_energy_rms(pair):
    syn, gs, w64, w32 = pair
    rng = np.random.default_rng(3)
    W = w64.nwalk
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, 3)), rng.uniform(size=(W, 1))], axis=-1)
    d = torch.as_tensor(dr, device=gs.device)
    e64, v64 = w64.lrdmc_energy(d, 0.2)
    e32, v32 = w32.lrdmc_energy(d, 0.2)
    de = (e32 - e64).cpu().numpy()
    rms = float(np.sqrt(np.mean(de**2)))
    print(f"{syn.name}: mixed vs fp64 e_L rms {rms:.3e} Ha, max {np.max(np.abs(de)):.3e}, mean {np.mean(de):.2e}")
    assert rms <= 1e-5
    assert abs(float(np.mean(de))) <= 1e-5


def test_mixed_projection_follows_fp64(pair):
    syn, gs, w64, w32 = pair
    from jqmc_gb300.engine import WalkerSet
    r = w64.r[:64].cpu().numpy()
    n = gs.n_up
    a = WalkerSet(gs, r[:, :n], r[:, n:], precision="fp64")
    b = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed")
    K = 20
    rng = np.random.default_rng(9)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (64, K, 3)), rng.uniform(size=(64, K, 1))], axis=-1)
    d = torch.as_tensor(dr, device=gs.device)
    wa = torch.ones(64, dtype=torch.float64, device=gs.device)
    wb = torch.ones_like(wa)
    a.lrdmc_project(d, 0.2, 0.0, wa)
    b.lrdmc_project(d, 0.2, 0.0, wb)
    torch.cuda.synchronize()
    same = (a.r - b.r).abs().amax(dim=(1, 2)) < 1e-6
    frac = float(same.double().mean())
    relw = ((wa - wb).abs() / wa.abs())[same]
    print(f"{syn.name}: {frac:.3f} of walkers on the same path; weight rel diff max {float(relw.max()):.2e}")
    assert frac >= 0.95
    assert float(relw.max()) < 5e-6 * K


def test_mixed_energy_after_block_and_rebuild(pair):
    """Production order of a branching cycle: K = 40 projections with float rank-1
    updates, the FP64 rebuild of the carried tables, then E_L.  On the walkers
    whose paths coincide with the FP64 form's, E_L meets the same bars as on
    freshly built tables."""
    syn, gs, w64, w32 = pair
    from jqmc_gb300.engine import WalkerSet
    r = w64.r.cpu().numpy()
    n = gs.n_up
    W = r.shape[0]
    a = WalkerSet(gs, r[:, :n], r[:, n:], precision="fp64")
    b = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed")
    K = 40
    rng = np.random.default_rng(17)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, K, 3)), rng.uniform(size=(W, K, 1))], axis=-1)
    d = torch.as_tensor(dr, device=gs.device)
    wa = torch.ones(W, dtype=torch.float64, device=gs.device)
    wb = torch.ones_like(wa)
    a.lrdmc_project(d, 0.2, 0.0, wa)
    b.lrdmc_project(d, 0.2, 0.0, wb)
    a.rebuild()
    b.rebuild()
    last = d[:, -1].contiguous()
    e64, _ = a.lrdmc_energy(last, 0.2)
    e32, _ = b.lrdmc_energy(last, 0.2)
    same = (a.r - b.r).abs().amax(dim=(1, 2)) < 1e-6
    de = (e32 - e64)[same].cpu().numpy()
    rms = float(np.sqrt(np.mean(de**2)))
    print(f"{syn.name}: after {K} projections + rebuild, e_L rms {rms:.3e} Ha on {len(de)} walkers, mean {np.mean(de):.2e}")
    assert float(same.double().mean()) >= 0.9
    assert rms <= 1e-5
    assert abs(float(np.mean(de))) <= 1e-5
    gi = (b.Ginv.double() - a.Ginv).abs().amax(dim=(1, 2)) / a.Ginv.abs().amax(dim=(1, 2))
    assert float(gi[same].max()) < 1e-5
    assert not b.status.any()


def test_mixed_gfmc_t_follows_fp64(pair):
    """GFMC_t projections with the same draws: the mixed form takes the same
    moves as the FP64 form for most walkers, with weights and spent time agreeing."""
    syn, gs, w64, w32 = pair
    from jqmc_gb300.engine import WalkerSet
    r = w64.r[:64].cpu().numpy()
    n = gs.n_up
    a = WalkerSet(gs, r[:, :n], r[:, n:], precision="fp64")
    b = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed")
    K = 40
    rng = np.random.default_rng(23)
    dr = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (64, K, 3)), rng.uniform(size=(64, K, 2))], axis=-1)
    d = torch.as_tensor(dr, device=gs.device)
    out = []
    for ws in (a, b):
        w = torch.ones(64, dtype=torch.float64, device=gs.device)
        tl = torch.full((64,), 0.01, dtype=torch.float64, device=gs.device)
        ns = torch.zeros(64, dtype=torch.int32, device=gs.device)
        el = torch.zeros(64, dtype=torch.float64, device=gs.device)
        ws.lrdmc_project_t(d, 0.2, w, tl, ns, el)
        out.append((w, tl, ns))
    same = (a.r - b.r).abs().amax(dim=(1, 2)) < 1e-6
    frac = float(same.double().mean())
    relw = ((out[0][0] - out[1][0]).abs() / out[0][0].abs())[same]
    print(f"{syn.name}: GFMC_t same path {frac:.3f}, weight rel diff max {float(relw.max()):.2e}")
    assert frac >= 0.9
    assert float(relw.max()) < 1e-4
    assert not b.status.any()


def test_mixed_fast_energy_variant(pair):
    """precision "mixed_fast_energy": the same float tables and projections, the
    block energy from float values with compensated float-float sums."""
    syn, gs, w64, w32 = pair
    from jqmc_gb300.engine import WalkerSet
    r = w64.r.cpu().numpy()
    n = gs.n_up
    we = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed_fast_energy")
    rng = np.random.default_rng(3)
    W = w64.nwalk
    d = torch.as_tensor(np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, 3)), rng.uniform(size=(W, 1))], axis=-1),
                        device=gs.device)
    e64, _ = w64.lrdmc_energy(d, 0.2)
    ee, _ = we.lrdmc_energy(d, 0.2)
    rms = float(torch.sqrt(torch.mean((ee - e64) ** 2)))
    print(f"{syn.name}: mixed tables + compensated float block energy vs fp64 e_L rms {rms:.3e} Ha")
    assert rms <= 1e-5
    assert torch.equal(we.Ginv, w32.Ginv)


def test_adaptive_block_energy(pair):
    """precision "mixed": the compensated-float energy; walkers whose mesh ratios
    cancel strongly (factor above the threshold) are recomputed in FP64
    arithmetic, the others keep the compensated value unchanged."""
    syn, gs, w64, w32 = pair
    from jqmc_gb300 import _lib
    from jqmc_gb300.engine import WalkerSet
    r = w64.r.cpu().numpy()
    n = gs.n_up
    we = WalkerSet(gs, r[:, :n], r[:, n:], precision="mixed_fast_energy")
    rng = np.random.default_rng(5)
    W = w64.nwalk
    d = torch.as_tensor(np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (W, 3)), rng.uniform(size=(W, 1))], axis=-1),
                        device=gs.device)
    e64, v64 = w64.lrdmc_energy(d, 0.2)
    ee, ve = we.lrdmc_energy(d, 0.2)
    ea, va = w32.lrdmc_energy(d, 0.2)
    cf = w32.energy_cancellation()
    flag = cf > _lib.FAST_ENERGY_CANCEL
    # sum |phi_a T_a| >= |sum phi_a T_a| element by element: the factor is at least 1
    assert bool(torch.isfinite(cf).all()) and float(cf.min()) >= 0.999
    assert float(flag.double().mean()) < 0.2
    # unflagged walkers: the compensated energy, bit for bit
    assert torch.equal(ea[~flag], ee[~flag]) and torch.equal(va[~flag], ve[~flag])
    rms = float(torch.sqrt(torch.mean((ea - e64) ** 2)))
    worst_flagged = float((ea - e64)[flag].abs().max()) if bool(flag.any()) else 0.0
    print(f"{syn.name}: adaptive block energy rms {rms:.3e} Ha, {int(flag.sum())}/{W} walkers recomputed in FP64 "
          f"(worst {worst_flagged:.3e} Ha), cancellation factor median {float(cf.median()):.2f}")
    assert rms <= 1e-5
    assert worst_flagged <= 5e-5
