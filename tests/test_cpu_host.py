"""CPU-only checks: the C ABI library and its exports, table packing, oracle
self-consistency, statistics, and the replica reduction across gloo ranks."""

import os
import re
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"^\s*(?:int|int32_t|int64_t)\s+(jqmc_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_loads_and_exports_every_declared_symbol():
    from jqmc_gb300 import _lib
    from jqmc_gb300.build import build
    build()
    import ctypes
    L = ctypes.CDLL(_lib.LIB_PATH)
    declared = _declared_symbols()
    assert len(declared) >= 14
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    assert set(_lib.EXPORTED) == set(declared)


@pytest.mark.parametrize("name", ["water_like", "ring12", "chain32"])
def test_pack_basis_covers_every_ao(name):
    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import pack_basis
    from oracle.ao import primitive_norm
    syn = synthetic.SYSTEMS[name]()
    g = syn.hamiltonian.wavefunction_data.geminal_data
    aos, _, _ = g.ao_basis_lambda()
    for basis in (aos, syn.hamiltonian.wavefunction_data.jastrow_data.jastrow_three_body_data.orb_data):
        shells, prims = pack_basis(basis)
        covered = np.zeros(basis.num_ao, dtype=int)
        for atom, l, npr, p0, ao0, nm, mf, _ in shells:
            covered[ao0:ao0 + nm] += 1
            for k in range(nm):
                assert basis.angular_momentums[ao0 + k] == l and basis.magnetic_quantum_numbers[ao0 + k] == mf + k
                assert basis.nucleus_index[ao0 + k] == atom
            z, c = basis.primitives_of(ao0)
            assert np.allclose(prims[p0:p0 + npr, 0], z)
            assert np.allclose(prims[p0:p0 + npr, 1], c * primitive_norm(l, z), rtol=1e-14)
        assert np.all(covered == 1)


def test_synthetic_workload_sizes():
    from jqmc_gb300 import synthetic
    w, r, c = synthetic.water_like(), synthetic.ring12(), synthetic.chain32()
    assert (w.n_up, w.n_dn) == (4, 4) and (r.n_up, r.n_dn) == (15, 15) and (c.n_up, c.n_dn) == (48, 48)
    aw = w.hamiltonian.wavefunction_data.geminal_data.ao_basis_lambda()[0].num_ao
    ar = r.hamiltonian.wavefunction_data.geminal_data.ao_basis_lambda()[0].num_ao
    ac = c.hamiltonian.wavefunction_data.geminal_data.ao_basis_lambda()[0].num_ao
    assert 35 <= aw <= 45 and 180 <= ar <= 220 and 650 <= ac <= 760
    assert r.hamiltonian.wavefunction_data.jastrow_data.jastrow_three_body_data.orb_num == 60


def test_oracle_sherman_morrison_stays_consistent():
    from jqmc_gb300 import synthetic
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.water_like()
    o = OracleSystem(syn.hamiltonian)
    ru, rd = syn.initial_electrons(1, seed=4)
    st = D.init_state(o, ru[0], rd[0])
    rng = np.random.default_rng(1)
    K = 60
    idr = np.stack([rng.integers(0, 8, K), rng.integers(0, 4, K), rng.integers(0, 4, K), rng.integers(0, 3, K)], 1)
    fdr = np.stack([rng.normal(size=K), rng.uniform(size=K)], 1)
    acc = D.vmc_block(o, st, idr, fdr, 0.4, 0.0)
    assert 0 < acc <= K
    G = o.geminal(st.r_up, st.r_dn)
    assert np.max(np.abs(st.G - G)) < 1e-10 * np.max(np.abs(G))
    assert np.max(np.abs(st.Ginv - np.linalg.inv(G))) < 1e-8 * np.max(np.abs(st.Ginv))


def test_oracle_branch_comb_semantics():
    from oracle.drivers import branch_comb
    w = np.array([1.0, 0.0, 3.0, 0.5])
    idx = branch_comb(w, 0.2)
    cum = np.cumsum(w / w.sum())
    z = (np.arange(4) + 0.2) / 4
    assert np.array_equal(idx, np.searchsorted(cum, z))
    assert 1 not in idx   # zero-weight walkers are never chosen


def test_jackknife_constant_energy():
    from jqmc_gb300.statistics import gfmc_G_L, jackknife_energy
    e = np.full((20, 3), -1.5)
    w = np.ones((20, 3))
    E, Es, V, Vs = jackknife_energy(e, e**2, w, 5)
    assert abs(E + 1.5) < 1e-14 and Es < 1e-12 and abs(V) < 1e-12
    g = gfmc_G_L(np.arange(1.0, 7.0).reshape(-1, 1), 2)
    assert np.allclose(g[:, 0], [1 * 2, 2 * 3, 3 * 4, 4 * 5])


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _replica_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    from jqmc_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    t = replicas.max_over_ranks(10.0 + rank)
    sums = torch.tensor([2.0 * (rank + 1), 1.0 + rank, -3.0 * (1.0 + rank), 9.0 * (1.0 + rank)], dtype=torch.float64)
    w_avg, e, e2 = replicas.lrdmc_observables(sums, num_walkers_per_rank=2)
    out.put((rank, t, w_avg, e, e2))
    dist.destroy_process_group()


def test_replica_reduction_gloo_world2():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, w_avg, e, e2 in res:
        assert t == 11.0
        assert abs(w_avg - (2.0 + 4.0) / 4) < 1e-15
        assert abs(e - (-3.0 - 6.0) / (1.0 + 2.0)) < 1e-15
        assert abs(e2 - (9.0 + 18.0) / 3.0) < 1e-15


def test_engine_refuses_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from jqmc_gb300 import synthetic
    from jqmc_gb300._lib import JqmcError
    from jqmc_gb300.engine import GpuSystem
    with pytest.raises(JqmcError):
        GpuSystem(synthetic.water_like().hamiltonian)


def test_jackknife_force_matches_direct_evaluation():
    """statistics.jackknife_force against a per-sample loop of the same estimator."""
    from jqmc_gb300.statistics import jackknife_force
    rng = np.random.default_rng(3)
    M, nw, na, bins = 20, 4, 2, 5
    w = rng.uniform(0.5, 1.5, (M, nw))
    e = rng.normal(-10, 1, (M, nw))
    fhf = rng.normal(0, 1, (M, nw, na, 3))
    fpp = rng.normal(0, 1, (M, nw, na, 3))
    efpp = e[..., None, None] * fpp
    mean, std = jackknife_force(w, e, fhf, fpp, efpp, bins)
    split = lambda x: [a.sum(axis=0) for a in np.array_split(x, bins, axis=0)]  # noqa: E731
    wb = np.concatenate(split(w))
    web = np.concatenate(split(w * e))
    fh = np.concatenate(split(w[..., None, None] * fhf))
    fp = np.concatenate(split(w[..., None, None] * fpp))
    ef = np.concatenate(split(w[..., None, None] * efpp))
    samples = []
    for j in range(len(wb)):
        W = wb.sum() - wb[j]
        E = (web.sum() - web[j]) / W
        FH = (fh.sum(0) - fh[j]) / W
        FP = (fp.sum(0) - fp[j]) / W
        EF = (ef.sum(0) - ef[j]) / W
        samples.append(-FH - 2.0 * (EF - E * FP))
    samples = np.array(samples)
    ref_mean = samples.mean(axis=0)
    ref_std = np.sqrt((len(samples) - 1) * np.mean((samples - ref_mean) ** 2, axis=0))
    assert np.allclose(mean, ref_mean, rtol=1e-12, atol=1e-12)
    assert np.allclose(std, ref_std, rtol=1e-12, atol=1e-12)


def test_entry_points_reject_invalid_arguments():
    """Every C-ABI entry point checks its handles, pointers and sizes before any
    CUDA call: null handles, null buffers and out-of-range sizes return
    JQMC_E_ARG (JQMC_E_LIMIT above a compiled maximum) without a device."""
    import ctypes as C

    from jqmc_gb300 import _lib
    from jqmc_gb300.build import build
    build()
    L = _lib.lib()
    E_ARG, E_LIMIT = -1, -2
    fake = C.c_void_p(0x100)          # never dereferenced: every call below fails its checks first
    w = _lib.Walkers()
    w.nwalk, w.precision = 4, _lib.PREC_FP64
    for f in ("r", "G", "Ginv", "Tup", "Tdn", "h3", "dphi", "dphi3", "ecache", "status"):
        setattr(w, f, fake)
    wp = C.byref(w)
    out = C.c_void_p()
    flops = C.c_double()
    calls = {
        "jqmc_system_create(desc=NULL)": L.jqmc_system_create(None, C.byref(out)),
        "jqmc_system_destroy(NULL)": L.jqmc_system_destroy(None),
        "jqmc_walker_bytes(NULL)": L.jqmc_walker_bytes(None, 0),
        "jqmc_ao_vgl(NULL)": L.jqmc_ao_vgl(None, 0, fake, 8, fake, None),
        "jqmc_walker_init(sys=NULL)": L.jqmc_walker_init(None, wp, None),
        "jqmc_lu_rebuild_refine(sys=NULL)": L.jqmc_lu_rebuild_refine(None, wp, None),
        "jqmc_log_psi(sys=NULL)": L.jqmc_log_psi(None, wp, fake, fake, fake, None),
        "jqmc_dlnpsi_dparam(sys=NULL)": L.jqmc_dlnpsi_dparam(None, wp, fake, fake, fake, None, None, None),
        "jqmc_dlnpsi_dR(sys=NULL)": L.jqmc_dlnpsi_dR(None, wp, fake, None),
        "jqmc_electron_terms(sys=NULL)": L.jqmc_electron_terms(None, wp, fake, None),
        "jqmc_kinetic_mesh(sys=NULL)": L.jqmc_kinetic_mesh(None, wp, fake, 0.2, fake, None),
        "jqmc_vmc_sweep(sys=NULL)": L.jqmc_vmc_sweep(None, wp, 4, fake, fake, 0.4, 0.0, fake, None),
        "jqmc_vmc_measure(sys=NULL)": L.jqmc_vmc_measure(None, wp, fake, 0.0, fake, fake, None),
        "jqmc_lrdmc_project(sys=NULL)": L.jqmc_lrdmc_project(None, wp, 4, fake, 0.2, 0.0, fake, None),
        "jqmc_lrdmc_energy(sys=NULL)": L.jqmc_lrdmc_energy(None, wp, fake, 0.2, fake, fake, None),
        "jqmc_lrdmc_project_t(sys=NULL)": L.jqmc_lrdmc_project_t(None, wp, 4, fake, 0.2, fake, fake, fake, fake, None),
        "jqmc_walker_gather(sys=NULL)": L.jqmc_walker_gather(None, wp, wp, fake, None),
        "jqmc_branch_comb(nwalk=0)": L.jqmc_branch_comb(0, fake, 0.5, fake, fake, None),
        "jqmc_branch_comb(zeta=1)": L.jqmc_branch_comb(8, fake, 1.0, fake, fake, None),
        "jqmc_branch_comb(w=NULL)": L.jqmc_branch_comb(8, None, 0.5, fake, fake, None),
        "jqmc_branch_comb_noalloc(nwalk=0)": L.jqmc_branch_comb_noalloc(0, fake, 0.5, fake, None),
        "jqmc_probe_fp64(iters=0)": L.jqmc_probe_fp64(0, 1, fake, C.byref(flops), None),
        "jqmc_probe_fp32(blocks=0)": L.jqmc_probe_fp32(10, 0, fake, C.byref(flops), None),
        "jqmc_batch_create(nitem=0)": L.jqmc_batch_create(0, None, None, C.byref(out)),
        "jqmc_batch_destroy(NULL)": L.jqmc_batch_destroy(None),
        "jqmc_batch_walkers(NULL)": L.jqmc_batch_walkers(None),
        "jqmc_vmc_sweep_batch(NULL)": L.jqmc_vmc_sweep_batch(None, 4, fake, fake, 0.4, 0.0, fake, 64, 0, None),
        "jqmc_vmc_sweep_batch(threads=33)": L.jqmc_vmc_sweep_batch(fake, 4, fake, fake, 0.4, 0.0, fake, 33, 0, None),
        "jqmc_batch_rebuild(NULL)": L.jqmc_batch_rebuild(None, 0, None),
        "jqmc_tensor_core_rebuild(NULL)": L.jqmc_tensor_core_rebuild(None),
    }
    bad = {k: v for k, v in calls.items() if v != E_ARG}
    assert not bad, bad
    # above the no-allocation comb's compiled maximum
    assert L.jqmc_branch_comb_noalloc(262145, fake, 0.5, fake, None) == E_LIMIT
    # every declared entry point is exercised above
    tested = {k.split("(")[0] for k in calls}
    assert tested == set(_lib.EXPORTED)


def test_drivers_keep_the_reference_signatures_and_refuse_unsupported_options():
    """MCMC / GFMC_n / GFMC_t take the reference's arguments in the reference's
    order (jqmc/jqmc_mcmc.py:129-143, jqmc/jqmc_gfmc.py:4222-4236 and :208-221),
    and refuse the options that are not on the GPU path before touching a GPU."""
    import inspect

    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n, GFMC_t
    from jqmc_gb300.jqmc_mcmc import MCMC
    ref = {
        MCMC: ["hamiltonian_data", "mcmc_seed", "num_walkers", "num_mcmc_per_measurement", "Dt", "epsilon_AS",
               "comput_log_WF_param_deriv", "comput_e_L_param_deriv", "comput_position_deriv",
               "random_discretized_mesh", "use_swct"],
        GFMC_n: ["hamiltonian_data", "num_walkers", "num_mcmc_per_measurement", "num_gfmc_collect_steps", "mcmc_seed",
                 "E_scf", "alat", "random_discretized_mesh", "non_local_move", "comput_position_deriv", "epsilon_PW",
                 "use_swct"],
        GFMC_t: ["hamiltonian_data", "num_walkers", "num_gfmc_collect_steps", "mcmc_seed", "tau", "alat",
                 "random_discretized_mesh", "non_local_move", "comput_position_deriv", "epsilon_PW", "use_swct"],
    }
    for cls, names in ref.items():
        params = list(inspect.signature(cls.__init__).parameters)[1:]
        assert params[:len(names)] == names, cls.__name__
    h = synthetic.water_like().hamiltonian
    with pytest.raises(NotImplementedError):
        MCMC(h, comput_e_L_param_deriv=True)
    with pytest.raises(NotImplementedError):
        GFMC_n(h, comput_position_deriv=True, use_swct=True)
    with pytest.raises(NotImplementedError):
        GFMC_t(h, comput_position_deriv=True, epsilon_PW=0.1)
    with pytest.raises(ValueError):
        GFMC_n(h, comput_position_deriv=True, precision="mixed")
    with pytest.raises(NotImplementedError):
        GFMC_t(h, non_local_move="dla")


def test_module_functions_keep_the_reference_names_and_need_a_gpu():
    """The module-level evaluation functions exist under the reference's names
    with its argument order; the RT -> Euler-angle inversion used by
    compute_local_energy reproduces the rotation; without a GPU they raise."""
    import inspect

    from jqmc_gb300 import (atomic_orbital, coulomb_potential, determinant, hamiltonians, jastrow_factor,
                            molecular_orbital, wavefunction)
    from jqmc_gb300._lib import JqmcError
    from jqmc_gb300.surface import angles_from_RT
    from oracle.wf import rotation_matrix
    expect = {
        atomic_orbital: {n: ["aos_data", "r_carts"] for n in
                         ("compute_AOs", "compute_AOs_grad", "compute_AOs_laplacian", "compute_AOs_value_grad_lap")},
        molecular_orbital: {n: ["mos_data", "r_carts"] for n in
                            ("compute_MOs", "compute_MOs_grad", "compute_MOs_laplacian", "compute_MOs_value_grad_lap")},
        determinant: {**{n: ["geminal_data", "r_up_carts", "r_dn_carts"] for n in
                         ("compute_geminal_all_elements", "compute_ln_det_geminal_all_elements",
                          "compute_det_geminal_all_elements", "compute_AS_regularization_factor",
                          "compute_grads_and_laplacian_ln_Det")},
                      "compute_AS_regularization_factor_fast_update": ["geminal", "geminal_inv"],
                      "compute_geminal_up_one_row_elements": ["geminal_data", "r_up_cart", "r_dn_carts"],
                      "compute_geminal_dn_one_column_elements": ["geminal_data", "r_up_carts", "r_dn_cart"],
                      "_compute_ratio_determinant_part_rank1_update": ["geminal_data", "A_old_inv", "old_r_up_carts",
                                                                       "old_r_dn_carts", "new_r_up_carts_arr",
                                                                       "new_r_dn_carts_arr"]},
        coulomb_potential: {**{n: ["coulomb_potential_data", "r_up_carts", "r_dn_carts"] for n in
                               ("compute_bare_coulomb_potential", "compute_bare_coulomb_potential_el_ion",
                                "compute_bare_coulomb_potential_el_ion_element_wise",
                                "compute_ecp_local_parts_all_pairs")},
                            "compute_bare_coulomb_potential_el_el": ["r_up_carts", "r_dn_carts"],
                            "compute_bare_coulomb_potential_ion_ion": ["coulomb_potential_data"],
                            "compute_coulomb_potential": ["coulomb_potential_data", "r_up_carts", "r_dn_carts", "RT",
                                                          "NN", "Nv", "wavefunction_data"],
                            "compute_ecp_coulomb_potential": ["coulomb_potential_data", "wavefunction_data", "r_up_carts",
                                                              "r_dn_carts", "RT", "NN", "Nv"]},
        jastrow_factor: {"compute_Jastrow_part": ["jastrow_data", "r_up_carts", "r_dn_carts"],
                         "_compute_ratio_Jastrow_part_rank1_update": ["jastrow_data", "old_r_up_carts", "old_r_dn_carts",
                                                                      "new_r_up_carts_arr", "new_r_dn_carts_arr", "j3_state"],
                         "compute_Jastrow_one_body": ["jastrow_one_body_data", "r_up_carts", "r_dn_carts"],
                         "compute_Jastrow_two_body": ["jastrow_two_body_data", "r_up_carts", "r_dn_carts"],
                         "compute_Jastrow_three_body": ["jastrow_three_body_data", "r_up_carts", "r_dn_carts"],
                         "compute_grads_and_laplacian_Jastrow_part": ["jastrow_data", "r_up_carts", "r_dn_carts"]},
        wavefunction: {**{n: ["wavefunction_data", "r_up_carts", "r_dn_carts"] for n in
                          ("evaluate_ln_wavefunction", "evaluate_wavefunction", "evaluate_jastrow",
                           "evaluate_determinant", "compute_kinetic_energy", "compute_kinetic_energy_all_elements")},
                       "evaluate_ln_wavefunction_fast": ["wavefunction_data", "r_up_carts", "r_dn_carts", "geminal_inv"],
                       "compute_discretized_kinetic_energy": ["alat", "wavefunction_data", "r_up_carts", "r_dn_carts", "RT"]},
        hamiltonians: {"compute_local_energy": ["hamiltonian_data", "r_up_carts", "r_dn_carts", "RT"],
                       "compute_local_energy_fast": ["hamiltonian_data", "r_up_carts", "r_dn_carts", "RT",
                                                     "geminal_inverse"]},
    }
    for mod, fns in expect.items():
        for name, args in fns.items():
            assert list(inspect.signature(getattr(mod, name)).parameters) == args, (mod.__name__, name)
    rng = np.random.default_rng(3)
    for a in rng.uniform(-2 * np.pi, 2 * np.pi, size=(20, 3)):
        RT = rotation_matrix(*a).T
        back = rotation_matrix(*angles_from_RT(RT)).T
        assert np.max(np.abs(back - RT)) < 1e-14
    with pytest.raises(ValueError):
        angles_from_RT(2.0 * np.eye(3))
    import torch
    if not torch.cuda.is_available():
        from jqmc_gb300 import synthetic
        syn = synthetic.water_like()
        aos = syn.hamiltonian.wavefunction_data.geminal_data.ao_basis_lambda()[0]
        with pytest.raises(JqmcError):
            atomic_orbital.compute_AOs(aos, np.zeros((2, 3)))


def test_system_descriptors_pass_the_library_validation():
    """The descriptors built for the workloads, for the TREXIO wavefunctions of
    the TurboRVB cases and for the stand-in Hamiltonians of the module-level
    functions pass jqmc_system_create's checks (on a machine without a GPU the
    call then stops at the device allocation: JQMC_E_CUDA)."""
    import ctypes as C

    from jqmc_gb300 import _lib, synthetic
    from jqmc_gb300.build import build
    from jqmc_gb300.engine import system_desc
    from jqmc_gb300.jastrow_factor import Jastrow_data
    from jqmc_gb300.surface import _ham_for_aos, _ham_for_jastrow, _ham_for_wavefunction
    build()
    L = _lib.lib()
    hams = []
    for name in ("water_like", "ring12", "chain32"):
        syn = synthetic.SYSTEMS[name]()
        wf = syn.hamiltonian.wavefunction_data
        jd = wf.jastrow_data
        hams += [(name, syn.hamiltonian), (name + "/aos", _ham_for_aos(wf.geminal_data.ao_basis_lambda()[0])),
                 (name + "/wavefunction", _ham_for_wavefunction(wf)),
                 (name + "/jastrow", _ham_for_jastrow(jd, syn.n_up, syn.n_dn)),
                 (name + "/j2", _ham_for_jastrow(Jastrow_data(jastrow_two_body_data=jd.jastrow_two_body_data),
                                                 syn.n_up, syn.n_dn))]
    from test_trexio import CASES, trexio_case
    for fixture, case in CASES:
        ham, _ = trexio_case(fixture, case)
        hams += [(f"{fixture}/{case}", ham), (f"{fixture}/{case}/wavefunction", _ham_for_wavefunction(ham.wavefunction_data))]
    for label, ham in hams:
        d, keep, _ = system_desc(ham)
        h = C.c_void_p()
        rc = L.jqmc_system_create(C.byref(d), C.byref(h))
        assert rc in (0, -3), (label, rc)    # JQMC_OK on a GPU machine, JQMC_E_CUDA without one
        if rc == 0:
            L.jqmc_system_destroy(h)


def test_bucket_assignment():
    """Electron-count buckets of the many-molecule batches: each molecule goes to
    the smallest bucket that holds it; above the largest bucket is an error."""
    from jqmc_gb300.batching import BUCKET_BOUNDS, bucket_of
    assert BUCKET_BOUNDS == tuple(sorted(BUCKET_BOUNDS))
    prev = 0
    for b in BUCKET_BOUNDS:
        assert bucket_of(prev + 1) == b and bucket_of(b) == b
        prev = b
    with pytest.raises(ValueError):
        bucket_of(BUCKET_BOUNDS[-1] + 1)


def test_as_factor_matches_the_oracle():
    """The Attaccalite-Sorella factor of the module-level functions (torch, any
    device) against the oracle's restatement, on random and singular matrices."""
    import torch

    from jqmc_gb300.surface import as_factor
    from oracle.wf import OracleSystem
    rng = np.random.default_rng(7)
    G = rng.normal(size=(6, 5, 5))
    G[3, 2] = 0.0                      # a zero row: the factor is 0, as the reference's where()
    Gi = np.stack([np.linalg.pinv(g) for g in G])
    got = as_factor(torch.as_tensor(G), torch.as_tensor(Gi)).numpy()
    want = np.array([OracleSystem.as_factor(g, gi) for g, gi in zip(G, Gi)])
    assert np.allclose(got, want, rtol=1e-14, atol=0.0), (got, want)
    assert got[3] == 0.0


def test_initial_electrons_follow_the_reference_assignment(golden_dir):
    """The nucleus of every initial electron equals the reference's
    _generate_init_electron_configurations on nine charge/spin cases
    (tests/golden/init_owners.npz); up electrons past the total charge go to
    random nuclei (per walker) in both; offsets lie between 0.1 and 1 bohr."""
    from jqmc_gb300._init_config import electron_owners, initial_electrons
    g = np.load(os.path.join(golden_dir, "init_owners.npz"))
    for name in g["cases"]:
        z, c, (nu, nd) = g[f"{name}.charges"], g[f"{name}.coords"], (int(x) for x in g[f"{name}.n"])
        up, dn, nr, order = electron_owners(z, c, nu, nd)
        ru, rd = g[f"{name}.up_owner"], g[f"{name}.dn_owner"]
        assert np.all(rd == dn[None]), name
        assert np.all(ru[:, :nu - nr] == up[None, :nu - nr]), name
        assert nr == 0 or not np.all(ru[:, nu - nr:] == ru[0, nu - nr:]), name    # random in the reference too
        r_up, r_dn = initial_electrons(c, z, nu, nd, 64, seed=3)
        assert r_up.shape == (64, nu, 3) and r_dn.shape == (64, nd, 3)
        d_dn = np.linalg.norm(r_dn - c[dn][None], axis=-1)
        assert np.all((d_dn >= 0.1) & (d_dn <= 1.0)), name
        near = np.min(np.linalg.norm(r_up[:, :, None, :] - c[None, None], axis=-1), axis=-1)
        assert np.all(near <= 1.0), name
        again = initial_electrons(c, z, nu, nd, 64, seed=3)
        assert np.array_equal(again[0], r_up) and np.array_equal(again[1], r_dn)
    with pytest.raises(ValueError):
        electron_owners(np.array([1.0]), np.zeros((1, 3)), 0, 2)


def test_rank1_row_column_and_ratio_algebra(golden_dir, monkeypatch):
    """The host algebra of compute_geminal_up_one_row_elements /
    _dn_one_column_elements and _compute_ratio_determinant_part_rank1_update
    (lambda folding, row/column assembly, rank-1 ratios) reproduces the
    reference's G and determinant ratios (tests/golden/water_like.npz) when the
    oracle's AO values stand in for the GPU AO call."""
    import torch

    from jqmc_gb300 import determinant as D
    from jqmc_gb300 import surface, synthetic
    from oracle.ao import AOTable, ao_value
    monkeypatch.setattr(surface, "ao_vgl",
                        lambda aos, r: torch.as_tensor(ao_value(AOTable(aos), np.asarray(r).reshape(-1, 3)))[None])
    g = np.load(os.path.join(golden_dir, "water_like.npz"))
    gem = synthetic.water_like().hamiltonian.wavefunction_data.geminal_data
    for w in range(g["r_up"].shape[0]):
        ru, rd, G = g["r_up"][w], g["r_dn"][w], g["geminal"][w]
        rows = np.stack([D.compute_geminal_up_one_row_elements(gem, ru[i:i + 1], rd) for i in range(len(ru))])
        cols = np.stack([D.compute_geminal_dn_one_column_elements(gem, ru, rd[j:j + 1]) for j in range(len(rd))], axis=1)
        np.testing.assert_allclose(rows, G, rtol=1e-12, atol=1e-14 * np.abs(G).max())
        np.testing.assert_allclose(cols, G, rtol=1e-12, atol=1e-14 * np.abs(G).max())
        nu, nd = [ru.copy()], [rd.copy()]       # the first configuration moves nothing: ratio 1
        for k in range(g["moves_spin"].shape[1]):
            u, d = ru.copy(), rd.copy()
            (u if g["moves_spin"][w, k] == 0 else d)[g["moves_idx"][w, k]] += g["moves_d"][w, k]
            nu.append(u)
            nd.append(d)
        r = D._compute_ratio_determinant_part_rank1_update(gem, np.linalg.inv(G), ru, rd, np.stack(nu), np.stack(nd))
        assert r[0] == 1.0
        np.testing.assert_allclose(r[1:], g["det_ratio"][w], rtol=1e-11)
    u2 = np.stack([ru + 0.1])
    with pytest.raises(ValueError):
        D._compute_ratio_determinant_part_rank1_update(gem, np.linalg.inv(G), ru, rd, u2, rd[None])


def test_nonlocal_move_option():
    """non_local_move reaches the system descriptor (T-move 0, dltmove 1); the
    library refuses any other code before touching the device, and the drivers
    accept both names."""
    import ctypes as C

    from jqmc_gb300 import _lib, synthetic
    from jqmc_gb300.build import build
    from jqmc_gb300.engine import system_desc
    from jqmc_gb300.jqmc_gfmc import _check_lrdmc_options
    build()
    L = _lib.lib()
    ham = synthetic.SYSTEMS["water_like"]().hamiltonian
    for name, code in (("tmove", 0), ("dltmove", 1)):
        d, keep, _ = system_desc(ham, 6, name)
        assert d.nonlocal_move == code
        h = C.c_void_p()
        assert L.jqmc_system_create(C.byref(d), C.byref(h)) in (0, -3)
        _check_lrdmc_options(name, False)
    d, keep, _ = system_desc(ham)
    d.nonlocal_move = 2
    h = C.c_void_p()
    assert L.jqmc_system_create(C.byref(d), C.byref(h)) == -1
    with pytest.raises(NotImplementedError):
        system_desc(ham, 6, "dla")
    with pytest.raises(NotImplementedError):
        _check_lrdmc_options("dla", False)


def test_cartesian_shell_table():
    """A Cartesian basis packs one shell per AO, {atom, l, nprim, prim0, ao, 1,
    component, 1}, with (Z, c N_cart) primitives; the library accepts it and
    refuses a bad kind or component index before touching the device."""
    import ctypes as C

    from cart_system import water_like_cartesian

    from jqmc_gb300 import _lib
    from jqmc_gb300.atomic_orbital import cartesian_norm, cartesian_orders
    from jqmc_gb300.build import build
    from jqmc_gb300.engine import pack_basis, system_desc
    build()
    L = _lib.lib()
    syn, ham = water_like_cartesian()
    aos = ham.wavefunction_data.geminal_data.orb_data_up_spin
    sh, pr = pack_basis(aos)
    assert sh.shape == (aos.num_ao, 8) and np.all(sh[:, 5] == 1) and np.all(sh[:, 7] == 1)
    for a in range(aos.num_ao):
        pw = (aos.polynominal_order_x[a], aos.polynominal_order_y[a], aos.polynominal_order_z[a])
        assert sh[a, 4] == a and cartesian_orders(int(sh[a, 1]))[sh[a, 6]] == pw
        z, c = aos.primitives_of(a)
        np.testing.assert_allclose(pr[sh[a, 3]:sh[a, 3] + sh[a, 2]],
                                   np.stack([z, c * np.array([cartesian_norm(int(sh[a, 1]), zz, *pw) for zz in z])], 1))
    d, keep, _ = system_desc(ham)
    h = C.c_void_p()
    assert L.jqmc_system_create(C.byref(d), C.byref(h)) in (0, -3)
    for col, bad in ((7, 2), (6, 99)):
        d, keep, _ = system_desc(ham)
        keep["dsh"][0, col] = bad
        assert L.jqmc_system_create(C.byref(d), C.byref(h)) == -1, (col, bad)
