"""Batches of molecules (jqmc_batch): one launch over the walkers of several
molecules against per-molecule launches, the mixed-precision batch against the
FP64 batch, and a captured CUDA graph against the same launches run eagerly."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SEEDS = (46, 7, 51)          # 4, 8 and 12 electrons
WALKERS = (32, 48, 40)


def _batch(precision, seed=3, buckets=False):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.batching import MoleculeBatch
    hams = [synthetic.random_molecule(s).hamiltonian for s in SEEDS]
    return MoleculeBatch(hams, WALKERS, precision=precision, seed=seed, buckets=buckets)


def _split(b, x):
    """per-molecule slices of a bucket-ordered walker array (one bucket)"""
    bk = b.buckets[0]
    return [x[bk.offsets[j]:bk.offsets[j + 1]] for j in range(len(bk.items))]


def test_fp64_batch_matches_single_molecule_sweeps():
    b = _batch("fp64")
    bk = b.buckets[0]
    idraw, fdraw = b.draws(bk, 12)
    # per-molecule launches with the same draws, on copies of the same walkers
    from jqmc_gb300.engine import WalkerSet
    singles = []
    for j, i in enumerate(bk.items):
        ws = b.walkers[i]
        n = b.systems[i].n_up
        r = ws.r.cpu().numpy()
        singles.append(WalkerSet(b.systems[i], r[:, :n], r[:, n:], precision="fp64"))
    acc_single = []
    for ws, idr, fdr in zip(singles, _split(b, idraw), _split(b, fdraw)):
        acc = torch.zeros(ws.nwalk, dtype=torch.int32, device=b.device)
        ws.vmc_sweep(idr.contiguous(), fdr.contiguous(), b.Dt, b.epsilon_AS, acc)
        acc_single.append(acc)
    r0 = [b.walkers[i].r.cpu().numpy().copy() for i in bk.items]
    b.sweep(bk, idraw, fdraw, caches=True, threads=64)
    torch.cuda.synchronize()
    for j, i in enumerate(bk.items):
        assert torch.equal(b.walkers[i].r, singles[j].r), f"molecule {i}"
        assert torch.equal(b.walkers[i].Ginv, singles[j].Ginv)
    assert torch.equal(bk.accept, torch.cat(acc_single))
    for ws in b.walkers:
        assert not ws.status.any()
    # and against the oracle (jqmc_mcmc.py:4278-4533): the first and last walker
    # of every molecule replayed with the batch's draws
    from jqmc_gb300 import synthetic
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    for j, (i, idr, fdr) in enumerate(zip(bk.items, _split(b, idraw), _split(b, fdraw))):
        o = OracleSystem(synthetic.random_molecule(SEEDS[i]).hamiltonian)
        n = o.n_up
        idr, fdr = idr.cpu().numpy(), fdr.cpu().numpy()
        for w in (0, WALKERS[i] - 1):
            st = D.init_state(o, r0[j][w, :n], r0[j][w, n:])
            D.vmc_block(o, st, idr[w], fdr[w], b.Dt, b.epsilon_AS)
            got = b.walkers[i].r[w].cpu().numpy()
            assert np.max(np.abs(got - np.vstack([st.r_up, st.r_dn]))) < 1e-12, (i, w)
    b.close()


def test_mixed_batch_follows_fp64_batch():
    a, m = _batch("fp64"), _batch("mixed")
    ba, bm = a.buckets[0], m.buckets[0]
    for wa, wm in zip(a.walkers, m.walkers):
        assert torch.equal(wa.r, wm.r)
    idraw, fdraw = a.draws(ba, 40)
    a.sweep(ba, idraw, fdraw, threads=64)
    m.sweep(bm, idraw, fdraw, threads=64)
    m.rebuild(False)
    torch.cuda.synchronize()
    same = torch.cat([(wa.r - wm.r).abs().amax(dim=(1, 2)) < 1e-6 for wa, wm in zip(a.walkers, m.walkers)])
    frac = float(same.double().mean())
    print(f"mixed batch on the FP64 batch's path: {frac:.3f}; accepted {int(bm.accept.sum())} vs {int(ba.accept.sum())}")
    assert frac >= 0.9
    for wa, wm in zip(a.walkers, m.walkers):
        keep = (wa.r - wm.r).abs().amax(dim=(1, 2)) < 1e-6
        rel = ((wm.Ginv.double() - wa.Ginv).abs().amax(dim=(1, 2)) / wa.Ginv.abs().amax(dim=(1, 2)))[keep]
        assert float(rel.max()) < 1e-4
        assert not wm.status.any()
    a.close()
    m.close()


def test_graph_replay_matches_eager_launches():
    g, e = _batch("mixed", buckets=True), _batch("mixed", buckets=True)
    tuned = g.autotune(K=4, candidates=(32, 64), reps=1)
    for bg, be in zip(g.buckets, e.buckets):
        be.threads = bg.threads
    # the autotuner moved g's walkers: give e the same positions and tables
    for wg, we in zip(g.walkers, e.walkers):
        we.r.copy_(wg.r)
    e.rebuild(True)
    g.rebuild(True)
    g.capture(steps=20, K=10)
    # e: the eager warm-up round the capture ran, then every round
    for b, (idraw, fdraw) in zip(e.buckets, g._draws[0]):
        e.sweep(b, idraw, fdraw)
    e.rebuild(False)
    for rnd in g._draws:
        for b, (idraw, fdraw) in zip(e.buckets, rnd):
            e.sweep(b, idraw, fdraw)
        e.rebuild(False)
    g.replay()
    torch.cuda.synchronize()
    for wg, we in zip(g.walkers, e.walkers):
        assert torch.equal(wg.r, we.r)
        assert torch.equal(wg.Ginv, we.Ginv)
    assert set(tuned) == {b.bound for b in g.buckets}
    assert g.graph_launches == 2 * len(g.buckets) * 3
    g.close()
    e.close()
