"""Host logic of the wavefunction optimisation (no GPU): the SR solve, the
generalized-force jackknife and the variational blocks.

The SR direction of jqmc_mcmc.py:2960-3345 is theta = D^-1/2 (D^-1/2 S D^-1/2 +
eps I)^-1 D^-1/2 f = (S + eps D)^-1 f with D = diag S; the tests check it
against that dense formula, whichever of the primal/dual systems and
direct/CG solves the routine takes.  The jackknife is checked against a
literal restatement of the reference's leave-one-out loops
(jqmc_mcmc.py:1541-1700)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _samples(M, nw, K, seed=0):
    rng = np.random.default_rng(seed)
    O = rng.normal(size=(M, nw, K)) * rng.uniform(0.1, 3.0, size=K)
    e = -1.0 + 0.3 * rng.normal(size=(M, nw)) + 0.2 * O[:, :, 0]
    w = rng.uniform(0.5, 1.0, size=(M, nw))
    return O, e, w


def _dense_sr(O, e, w, eps):
    O = O.reshape(-1, O.shape[-1])
    e, w = e.ravel(), w.ravel()
    Wt = w.sum()
    dO = O - (w @ O) / Wt
    de = e - (w @ e) / Wt
    S = (dO * w[:, None]).T @ dO / Wt
    f = -2.0 * (dO * w[:, None]).T @ de / Wt
    return np.linalg.solve(S + eps * np.diag(np.diag(S)), f), f


@pytest.mark.parametrize("M,nw,K", [(20, 8, 5), (3, 4, 30)])        # fewer / more parameters than samples
@pytest.mark.parametrize("cg", [False, True])
def test_sr_direction_matches_dense_solve(M, nw, K, cg):
    from jqmc_gb300.variational import sr_direction
    O, e, w = _samples(M, nw, K)
    eps = 1e-3
    ref, f = _dense_sr(O, e, w, eps)
    r = sr_direction(O, e, w, eps, cg_flag=cg, cg_tol=1e-13)
    np.testing.assert_allclose(r.f, f, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(r.theta, ref, rtol=1e-7, atol=1e-9 * np.max(np.abs(ref)))
    assert not r.frozen.any()
    if cg:
        assert r.cg_iterations > 0 and r.warm_start is not None
        again = sr_direction(O, e, w, eps, cg_flag=True, cg_tol=1e-13, warm_start=r.warm_start)
        assert again.cg_iterations <= 1
        np.testing.assert_allclose(again.theta, r.theta, rtol=1e-9, atol=1e-12)


def test_sr_direction_freezes_constant_parameters():
    """A parameter whose derivative does not vary has diag S = 0: it is frozen
    (theta 0) and the others solve the system without it."""
    from jqmc_gb300.variational import sr_direction
    O, e, w = _samples(30, 6, 4, seed=3)
    O[:, :, 2] = 0.7
    r = sr_direction(O, e, w, 1e-3, cg_flag=False)
    assert r.frozen.tolist() == [False, False, True, False] and r.theta[2] == 0.0
    keep = [0, 1, 3]
    ref, _ = _dense_sr(O[:, :, keep], e, w, 1e-3)
    np.testing.assert_allclose(r.theta[keep], ref, rtol=1e-9)


def test_sr_direction_rejects_mismatched_samples():
    from jqmc_gb300.variational import sr_direction
    O, e, w = _samples(4, 3, 2)
    with pytest.raises(ValueError):
        sr_direction(O, e[:-1], w[:-1], 1e-3)


def _jackknife_loops(w_L, e_L, O, bins):
    """The leave-one-out loops of jqmc_mcmc.py:1541-1700 written out."""
    ws = np.array_split(w_L, bins, axis=0)
    wes = np.array_split(w_L * e_L, bins, axis=0)
    wOs = np.array_split(w_L[:, :, None] * O, bins, axis=0)
    weOs = np.array_split((w_L * e_L)[:, :, None] * O, bins, axis=0)
    wb = [x for a in ws for x in a.sum(axis=0)]
    web = [x for a in wes for x in a.sum(axis=0)]
    wOb = [x for a in wOs for x in a.sum(axis=0)]
    weOb = [x for a in weOs for x in a.sum(axis=0)]
    W, WE, WO, WEO = sum(wb), sum(web), sum(wOb), sum(weOb)
    fj = []
    for j in range(len(wb)):
        d = W - wb[j]
        fj.append(-2.0 * ((WEO - weOb[j]) / d - ((WE - web[j]) / d) * ((WO - wOb[j]) / d)))
    fj = np.array(fj)
    mean = fj.mean(axis=0)
    return mean, np.sqrt((len(fj) - 1) * np.mean((fj - mean) ** 2, axis=0))


def test_generalized_force_jackknife_matches_the_reference_loops():
    from jqmc_gb300.statistics import jackknife_generalized_force
    O, e, w = _samples(23, 5, 6, seed=1)
    m, s = jackknife_generalized_force(w, e, O, 4)
    rm, rs = _jackknife_loops(w, e, O, 4)
    np.testing.assert_allclose(m, rm, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(s, rs, rtol=1e-10)
    _, f = _dense_sr(O, e, w, 1e-3)
    np.testing.assert_allclose(m, f, rtol=0.05, atol=0.02)   # the jackknife mean is close to the plain estimate
    with pytest.raises(ValueError):
        jackknife_generalized_force(w[:3], e[:3], O[:3], 4)


def _wavefunction(sym_j3=True, sym_lambda=True):
    from jqmc_gb300 import synthetic
    import dataclasses
    wf = synthetic.SYSTEMS["water_like"]().hamiltonian.wavefunction_data
    rng = np.random.default_rng(5)
    j3 = wf.jastrow_data.jastrow_three_body_data
    jm = np.array(j3.j_matrix)
    if not sym_j3:
        jm[0, 1] += 0.3
    lam = np.array(wf.geminal_data.lambda_matrix)
    lam = 0.5 * (lam + lam.T) if sym_lambda else lam + np.triu(rng.normal(size=lam.shape), 1)
    jd = dataclasses.replace(wf.jastrow_data, jastrow_three_body_data=dataclasses.replace(j3, j_matrix=jm))
    return dataclasses.replace(wf, jastrow_data=jd, geminal_data=dataclasses.replace(wf.geminal_data, lambda_matrix=lam))


def test_variational_blocks_and_updates_keep_the_symmetries():
    from jqmc_gb300.variational import apply_block_updates, get_variational_blocks
    wf = _wavefunction()
    jm0 = wf.jastrow_data.jastrow_three_body_data.j_matrix
    assert np.allclose(jm0[:, :-1], jm0[:, :-1].T)
    blocks = get_variational_blocks(wf, opt_lambda_param=True)
    names = [b.name for b in blocks]
    assert names == [n for n in ("j1_param", "j2_param", "j3_matrix", "lambda_matrix")
                     if n != "j1_param" or wf.jastrow_data.jastrow_one_body_data is not None]
    K = sum(b.size for b in blocks)
    theta = np.random.default_rng(2).normal(size=K)
    new = apply_block_updates(wf, blocks, theta, 0.01)
    jm = new.jastrow_data.jastrow_three_body_data.j_matrix
    lam = new.geminal_data.lambda_matrix
    np.testing.assert_array_equal(jm[:, :-1], jm[:, :-1].T)
    np.testing.assert_array_equal(lam, lam.T)
    pos = {b.name: sum(c.size for c in blocks[:i]) for i, b in enumerate(blocks)}
    assert new.jastrow_data.jastrow_two_body_data.jastrow_2b_param == pytest.approx(
        wf.jastrow_data.jastrow_two_body_data.jastrow_2b_param + 0.01 * theta[pos["j2_param"]])
    # the last J3 column (the one-body part) moves freely
    a3 = jm.shape[0]
    t3 = theta[pos["j3_matrix"]:pos["j3_matrix"] + jm.size].reshape(jm.shape)
    np.testing.assert_allclose(jm[:, a3], jm0[:, a3] + 0.01 * t3[:, a3])
    # the symmetry callbacks symmetrise sample rows the same way
    b3 = blocks[names.index("j3_matrix")]
    rows = np.random.default_rng(4).normal(size=(3, b3.size))
    sym = b3.symmetrize_metric(rows).reshape(3, *b3.shape)
    np.testing.assert_array_equal(sym[:, :, :a3], np.swapaxes(sym[:, :, :a3], 1, 2))
    # a zero slice leaves its block untouched (the same object)
    zero = np.zeros(K)
    same = apply_block_updates(wf, blocks, zero, 1.0)
    assert same.jastrow_data.jastrow_three_body_data is wf.jastrow_data.jastrow_three_body_data


def test_non_symmetric_matrices_are_not_symmetrised():
    from jqmc_gb300.variational import apply_block_updates, get_variational_blocks
    wf = _wavefunction(sym_j3=False, sym_lambda=False)
    blocks = get_variational_blocks(wf, opt_J1_param=False, opt_J2_param=False, opt_lambda_param=True)
    assert [b.name for b in blocks] == ["j3_matrix", "lambda_matrix"]
    theta = np.random.default_rng(6).normal(size=sum(b.size for b in blocks))
    new = apply_block_updates(wf, blocks, theta, 0.1)
    jm = new.jastrow_data.jastrow_three_body_data.j_matrix
    n3 = blocks[0].size
    np.testing.assert_allclose(jm.ravel(), wf.jastrow_data.jastrow_three_body_data.j_matrix.ravel() + 0.1 * theta[:n3])
    np.testing.assert_allclose(new.geminal_data.lambda_matrix.ravel(),
                               wf.geminal_data.lambda_matrix.ravel() + 0.1 * theta[n3:])


def test_variational_block_options():
    from jqmc_gb300.variational import apply_block_updates, get_variational_blocks
    wf = _wavefunction()
    assert "lambda_matrix" not in [b.name for b in get_variational_blocks(wf)]
    with pytest.raises(NotImplementedError):
        get_variational_blocks(wf, opt_J3_basis_exp=True)
    blocks = get_variational_blocks(wf)
    with pytest.raises(ValueError):
        apply_block_updates(wf, blocks, np.zeros(3), 1.0)


def test_wavefunction_methods_are_the_module_functions():
    from jqmc_gb300.variational import get_variational_blocks
    wf = _wavefunction()
    a = wf.get_variational_blocks(opt_lambda_param=True)
    b = get_variational_blocks(wf, opt_lambda_param=True)
    assert [x.name for x in a] == [x.name for x in b]
    theta = np.linspace(-1.0, 1.0, sum(x.size for x in a))
    new = wf.apply_block_updates(a, theta, 0.01)
    np.testing.assert_allclose(new.geminal_data.lambda_matrix, new.geminal_data.lambda_matrix.T)


def test_run_optimize_loop_converges_on_a_linear_energy_model():
    """run_optimize's host loop with a stand-in for the walker kernels.  The
    stand-in draws derivatives O and sets e_L = E0 + O_sym . (c - c*) / 2
    exactly (O_sym the block-symmetrised O), so cov(O, e_L) = S (c - c*) / 2, f =
    -S (c - c*) and the SR direction is theta = -(c - c*) up to the epsilon
    shift: each step of size delta must shrink c - c* by (1 - delta).  Checks
    the signs, the block order and symmetry, and the sampler reset."""
    import dataclasses
    import types

    from jqmc_gb300.hamiltonians import Hamiltonian_data
    from jqmc_gb300.jqmc_mcmc import MCMC
    from jqmc_gb300.variational import get_variational_blocks
    from jqmc_gb300 import synthetic

    ham0 = synthetic.SYSTEMS["water_like"]().hamiltonian
    wf0 = _wavefunction()
    ham0 = dataclasses.replace(ham0, wavefunction_data=wf0)
    flags = dict(opt_J1_param=False)
    target = {b.name: np.array(b.values, dtype=np.float64) for b in get_variational_blocks(wf0, **flags)}
    rng = np.random.default_rng(11)
    target["j2_param"] = target["j2_param"] + 0.4
    t3 = rng.normal(scale=0.05, size=target["j3_matrix"].shape)
    t3[:, :-1] = 0.5 * (t3[:, :-1] + t3[:, :-1].T)
    target["j3_matrix"] = target["j3_matrix"] + t3
    W, M_per_step = 64, 40

    m = MCMC.__new__(MCMC)
    m.num_walkers = W
    m.comput_log_WF_param_deriv = True
    m.comput_position_deriv = False
    m._opt_lambda = True
    m.sys = types.SimpleNamespace(device=torch.device("cpu"), n_up=4)
    m.walkers = types.SimpleNamespace(r=torch.zeros((W, 8, 3), dtype=torch.float64))
    resets = []

    def build(ham, r_up, r_dn, seed=0):
        m._hamiltonian_data = ham
        m._e_L, m._w_L, m._param_grads = [], [], {}
        m.mcmc_counter = 0
        resets.append(r_up.shape)

    def run(num_mcmc_steps=0, max_time=86400):
        blocks = get_variational_blocks(m.hamiltonian_data.wavefunction_data, **flags)
        v = np.concatenate([(np.asarray(b.values) - target[b.name]).ravel() / 2.0 for b in blocks])
        for _ in range(num_mcmc_steps):
            parts, sym = [], []
            for b in blocks:
                o = rng.normal(size=(W, b.size))
                parts.append(o)
                sym.append(b.symmetrize_metric(o) if b.symmetrize_metric is not None else o)
            e = -17.0 + np.concatenate(sym, axis=1) @ v
            m._e_L.append(e)
            m._w_L.append(np.ones(W))
            for b, o in zip(blocks, parts):
                m._param_grads.setdefault(b.name, []).append(o.reshape((W,) + tuple(b.shape)))
            m.mcmc_counter += 1

    m._build = build
    m.run = run
    build(ham0, np.zeros((W, 4, 3)), np.zeros((W, 4, 3)))
    resets.clear()

    def err(wf):
        return np.concatenate([(np.asarray(b.values) - target[b.name]).ravel()
                               for b in get_variational_blocks(wf, **flags)])

    e0 = np.linalg.norm(err(wf0))
    delta = 0.5
    hist = m.run_optimize(num_mcmc_steps=M_per_step, num_opt_steps=3, num_mcmc_warmup_steps=0, num_mcmc_bin_blocks=5,
                          optimizer_kwargs=dict(delta=delta, epsilon=1e-6, cg_flag=False), **flags)
    assert len(hist) == 3 and len(resets) == 3 and m.mcmc_counter == 0
    assert all(h["frozen"] == 0 and np.isfinite(h["E"]) for h in hist)
    wf3 = m.hamiltonian_data.wavefunction_data
    ratio = np.linalg.norm(err(wf3)) / e0
    assert abs(ratio - (1 - delta) ** 3) < 0.01 * (1 - delta) ** 3, ratio
    jm = wf3.jastrow_data.jastrow_three_body_data.j_matrix
    np.testing.assert_array_equal(jm[:, :-1], jm[:, :-1].T)
    # the same loop through the CG solver
    m.hamiltonian_data = ham0
    m.run_optimize(num_mcmc_steps=M_per_step, num_opt_steps=1, num_mcmc_warmup_steps=0, num_mcmc_bin_blocks=5,
                   optimizer_kwargs=dict(delta=delta, epsilon=1e-6, cg_tol=1e-12, cg_max_iter=20000), **flags)
    ratio = np.linalg.norm(err(m.hamiltonian_data.wavefunction_data)) / e0
    assert abs(ratio - (1 - delta)) < 0.01 * (1 - delta), ratio
    with pytest.raises(NotImplementedError):
        m.run_optimize(num_opt_steps=1, optimizer_kwargs=dict(method="adam"))
    with pytest.raises(RuntimeError):
        m.run_optimize(num_opt_steps=1, optimizer_kwargs=dict(use_lm=True))
