"""Walker-path benchmark on GB300: LRDMC (GFMC_n) projections, mixed precision vs plain FP64.

Workload (default, --workload chain32): the 32-nucleus zig-zag chain -- 16
C-like nuclei (Z_eff 4, semilocal ECP with l = 0, 1 non-local channels) and 16
H, bond 2.6 bohr, 96 electrons (48/48), 736 spherical GTOs, JAGP geminal,
J1/J2/J3 (64 J3 AOs); 16384 walkers; lattice spacing 0.2 bohr, 6 directions;
T-move ECP (Nv = 6); 40 projections per branching.  (--workload ring12: the
12-nucleus ring, 30 electrons, 192 AOs, 8192 walkers.)  One bench step = one
branching cycle: 40 projections of every walker, the FP64 rebuild of G^-1 / T
tables from the positions (LU + one refinement step), the local energy, the
weighted sums and the comb reconfiguration.  walker-steps per bench step = walkers x 40.  The plain FP64 arm
runs the same draws for fewer cycles (min(warmup, 1) + max(1, steps // 2)).

value : walker-steps/s of the mixed-precision form with the draws resident in
        HBM; the plain FP64 form runs the same draws and is reported beside it
        (plain_fp64, speedup_vs_plain_fp64) with the accuracy of the mixed form
        against it (per-configuration e_L rms, difference of mean energies).
e2e   : the mixed form through the public driver API (jqmc_gb300.jqmc_gfmc.GFMC_n.run_block)
        with the draws copied from pinned host memory each step and the step's
        sums read back to the host.
Walker state is several GB (> L2, 129 MB), so no L2 flush is needed.

Further legs in the same line (rank 0; skipped with --no-adjoint,
--no-batching, --no-vmc):
adjoint  : per-walker d ln psi / d theta on ring12 (8192 walkers).
batching : 64 molecules of uneven size, mixed VMC in one CUDA graph per
           electron-count bucket, against sequential per-molecule FP64 launches.
vmc      : VMC on the chain (16384 walkers), mixed batched sweep with its
           drift-control rebuild against the same sweep in FP64, same draws.

--impl reference : the CPU oracle (NumPy restatement of the reference, which is
Python/JAX and cannot run without JAX) on all host cores, one process per core,
each projecting its own walker; a bounded sample per step.
"""

from __future__ import annotations

import argparse
import copy
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s on 1 GB300: mixed-prec+batched vs plain FP64 at |Δ<E>|≤0.1 mHa"
NCU_TRAFFIC_PER_WALKER_STEP = {"chain32": (5.096144e9 + 0.7726876e9) / (912 * 2)}
UNIT = "walker-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="chain32", choices=["ring12", "water_like", "chain32"])
    p.add_argument("--walkers", type=int, default=None, help="default: 16384 for chain32, 8192 otherwise")
    p.add_argument("--nproj", type=int, default=40)
    p.add_argument("--alat", type=float, default=0.2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-adjoint", action="store_true", help="skip the parameter-derivative leg")
    p.add_argument("--no-batching", action="store_true", help="skip the many-molecule leg")
    p.add_argument("--no-vmc", action="store_true", help="skip the chain32 VMC leg (mixed vs plain FP64)")
    p.add_argument("--no-configs", action="store_true", help="skip the config 0 (VMC water) and config 1 (LRDMC ring12) legs")
    a = p.parse_args()
    if a.walkers is None:
        a.walkers = 16384 if a.workload == "chain32" else 8192
    return a


# ----------------------------------------------------------------------------- CPU oracle arm
def _oracle_worker(args):
    """Run branching cycles of the walker-batched NumPy GFMC_n step (oracle/batched.py:
    the oracle's algorithm with every mesh point of a walker in one array): K
    projections, then the block energy, as the GPU cycle does (the comb over one
    process's walkers is left out: it costs nothing next to a projection).  Whole
    cycles until about `budget` seconds have passed, after one untimed step;
    returns walker-steps done and seconds."""
    workload, seed, alat, budget, walkers, K = args
    from jqmc_gb300 import synthetic
    from oracle.batched import BatchedGFMCn
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[workload]()
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(walkers, seed=seed)
    r = np.concatenate([r_up, r_dn], axis=1)
    b = BatchedGFMCn(o, alat)
    rng = np.random.default_rng(seed)
    w = np.ones(walkers)

    def draws():
        return np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, (walkers, 3)), rng.uniform(size=(walkers, 1))], axis=1)

    r, w, _, _, _ = b.step(r, w, draws(), 0.0)
    t0 = time.perf_counter()
    done = 0
    while True:
        for _ in range(K):
            d = draws()
            r, w, _, _, _ = b.step(r, w, d, 0.0)
        b.energy(r, d)
        w[:] = 1.0
        done += walkers * K
        if time.perf_counter() - t0 >= budget:
            break
    return done, time.perf_counter() - t0


def oracle_rate(workload: str, alat: float, procs: int, budget: float, K: int = 40, walkers: int = 1):
    """walker-steps/s of the batched NumPy cycle with `procs` single-threaded
    processes (spawned before any GPU use), each projecting its own walkers."""
    if procs == 1:
        done, secs = _oracle_worker((workload, 0, alat, budget, walkers, K))
        return done / secs, done
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:   # the spawned workers start with one BLAS thread each
        os.environ[k] = "1"
    try:
        with ctx.Pool(procs) as pool:
            res = pool.map(_oracle_worker, [(workload, s, alat, budget, walkers, K) for s in range(procs)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return sum(d / s for d, s in res), sum(d for d, _ in res)


def _vmc_worker(args):
    """VMC blocks of the walker-batched NumPy Metropolis step (oracle/batched.py
    BatchedVMC): K proposals of every walker, then E_L and w_L, whole blocks for
    about `budget` seconds after one untimed proposal; returns walker-steps
    (proposals) done and seconds."""
    workload, seed, budget, walkers, K = args
    from jqmc_gb300 import synthetic
    from oracle.batched import BatchedVMC
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[workload]()
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(walkers, seed=seed)
    r = np.concatenate([r_up, r_dn], axis=1)
    b = BatchedVMC(o, 0.4, 0.0)
    G, Ginv = b.init(r)
    rng = np.random.default_rng(seed)
    n, nd = o.n_up, o.n_dn

    def draws():
        idraw = np.stack([rng.integers(0, n + nd, walkers), rng.integers(0, n, walkers), rng.integers(0, max(nd, 1), walkers),
                          rng.integers(0, 3, walkers)], axis=-1)
        return idraw, np.stack([rng.normal(size=walkers), rng.uniform(size=walkers)], axis=-1)

    b.proposal(r, G, Ginv, *draws())
    t0 = time.perf_counter()
    done = 0
    while True:
        for _ in range(K):
            b.proposal(r, G, Ginv, *draws())
        b.measure(r, G, Ginv, rng.uniform(-np.pi, np.pi, (walkers, 3)))
        done += walkers * K
        if time.perf_counter() - t0 >= budget:
            break
    return done, time.perf_counter() - t0


def vmc_cpu_rate(workload: str, procs: int, budget: float, K: int = 40, walkers: int = 64):
    """walker-steps/s (proposals) of the batched NumPy VMC blocks with `procs`
    single-threaded processes, each with its own walkers."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = "1"
    try:
        with ctx.Pool(procs) as pool:
            res = pool.map(_vmc_worker, [(workload, s, budget, walkers, K) for s in range(procs)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return sum(d / s for d, s in res), sum(d for d, _ in res)


def reference_arm(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    vals = []
    budget = 15.0
    for _ in range(a.steps):
        v, _ = oracle_rate(a.workload, a.alat, cores, budget, a.nproj)
        vals.append(v)
    v = statistics.median(vals)
    sample = (f"{cores} single-threaded processes x 1 walker of {a.workload}, branching cycles of {a.nproj} "
              f"walker-batched NumPy GFMC_n steps and the block energy (oracle/batched.py), whole cycles for "
              f"at least {budget:.0f} s after one untimed step, median of {a.steps} samples")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": f"lrdmc_{a.workload}", "walkers": a.walkers, "projections_per_branching": a.nproj,
                                             "alat": a.alat, "parallelism": "host processes"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Python/JAX; JAX is not installed, so the CPU oracle port stands in"}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.idx = device_index
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={device_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- GPU arm
def _probe(L, fn, dev, stream, dtype):
    import ctypes

    import torch
    sink = torch.zeros(1, dtype=dtype, device=dev)
    fl = ctypes.c_double()
    blocks = torch.cuda.get_device_properties(dev).multi_processor_count * 8
    fn(2000, blocks, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(fl), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn(20000, blocks, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(fl), ctypes.c_void_p(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    return fl.value / (e0.elapsed_time(e1) / 1e3) / 1e9


def _time_form(drv, draws, zetas, warmup, steps, stream, world, dev):
    """Warm up, then time `steps` branching cycles with device-resident draws.
    Returns (ms, per-step sums (steps, 4), list of project-launch ms, list of rebuild-launch ms)."""
    import torch
    import torch.distributed as dist

    from jqmc_gb300.replicas import max_over_ranks
    cls = drv.walkers.__class__
    orig, orig_rb = cls.lrdmc_project, cls.rebuild
    events, events_rb = [], []

    def timed_project(self, d, alat, E_scf, w):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        orig(self, d, alat, E_scf, w)
        e1.record(stream)
        events.append((e0, e1))

    def timed_rebuild(self):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        orig_rb(self)
        e1.record(stream)
        events_rb.append((e0, e1))

    for s in range(warmup):
        drv.run_block(draws[s], zetas[s])
    torch.cuda.synchronize()
    cls.lrdmc_project = timed_project
    cls.rebuild = timed_rebuild
    try:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        sums = [drv.run_block(draws[s], zetas[s]) for s in range(warmup, warmup + steps)]
        t1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    finally:
        cls.lrdmc_project, cls.rebuild = orig, orig_rb
    ms = max_over_ranks(t0.elapsed_time(t1), device=dev)
    return (ms, torch.stack(sums).cpu().numpy(), [a.elapsed_time(b) for a, b in events],
            [a.elapsed_time(b) for a, b in events_rb])


def adjoint_leg(stream, dev, peak64, hbm_peak, walkers: int = 8192, reps: int = 5):
    """Parameter derivatives of ln|psi| (J1, J2, J3 block, lambda block) on the
    12-nucleus ring with 8192 walkers: one jqmc_dlnpsi_dparam launch per rep."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.adjoint import dlnpsi_dparams
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from jqmc_gb300.workload import dlnpsi_bytes, dlnpsi_flops
    syn = synthetic.ring12()
    gs = GpuSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(walkers, seed=77)
    ws = WalkerSet(gs, r_up, r_dn)
    for _ in range(3):
        blocks = dlnpsi_dparams(ws)
    del blocks
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        blocks = dlnpsi_dparams(ws)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        del blocks
    t = statistics.median(ms)
    fl = dlnpsi_flops(gs) * walkers
    by = dlnpsi_bytes(gs) * walkers
    out = {"workload": "ring12 d ln psi / d (j1, j2, j3_matrix 60x61, lambda 192x192), FP64", "walkers": walkers,
           "ms": t, "walker_derivatives_per_s": walkers / (t / 1e3),
           "fp64_gflops": fl / (t / 1e3) / 1e9, "fp64_peak": peak64, "fp64_frac": fl / (t / 1e3) / 1e9 / peak64,
           "hbm_gbs": by / (t / 1e3) / 1e9, "hbm_peak": hbm_peak,
           "note": "CUDA events around dlnpsi_dparams (one kernel launch, blocks allocated by the caller); median of 5"}
    del ws, gs
    torch.cuda.empty_cache()
    return out


def forces_leg(stream, walkers: int = 8192):
    """Config 3's forces on the 12-nucleus ring with 8192 walkers: d ln psi/dR
    (one jqmc_dlnpsi_dR launch) and dE_L/dR by five-point differences of the
    FP64 VMC local energy (12 natom displaced systems, built once, each a walker
    initialisation and an E_L launch per call)."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.engine import GpuSystem, WalkerSet
    from jqmc_gb300.forces import ELGradientFD, dlnpsi_dR
    syn = synthetic.ring12()
    gs = GpuSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(walkers, seed=78)
    ws = WalkerSet(gs, r_up, r_dn)
    angles = torch.as_tensor(np.random.default_rng(5).uniform(-np.pi, np.pi, (walkers, 3)), device=gs.device)
    fd = ELGradientFD(syn.hamiltonian)
    dlnpsi_dR(ws)
    torch.cuda.synchronize()

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    ms_psi, _ = timed(lambda: dlnpsi_dR(ws))
    ms_el, g = timed(lambda: fd(r_up, r_dn, angles))
    finite = bool(torch.isfinite(g).all())
    out = {"workload": "ring12 forces (12 nuclei, 30 electrons), FP64", "walkers": walkers,
           "dlnpsi_dR_ms": ms_psi, "dEL_dR_ms": ms_el, "el_evaluations_per_walker": 12 * int(fd.M),
           "walker_forces_per_s": walkers / ((ms_psi + ms_el) / 1e3), "finite": finite,
           "note": "CUDA events; dE_L/dR by differences of the GPU E_L (4 displaced systems per nucleus and axis), "
                   "d ln psi/dR analytic (one launch); the displaced systems are created before timing"}
    del ws, gs, fd
    torch.cuda.empty_cache()
    return out


def batching_leg(nmol: int = 64, steps: int = 500, K: int = 50, fp64_steps: int = 50):
    """64 independent molecules (1-20 nuclei, Z_eff in {1, 4, 6}), walkers in
    proportion to the electron count (256-4096), VMC in the mixed precision:
    one CUDA graph of batched launches per electron-count bucket (CTA size
    autotuned per bucket), table rebuild every K proposals; against sequential
    per-molecule launches of the plain FP64 form with the same work per proposal
    (neither keeps the energy caches current between measurements)."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.batching import MoleculeBatch
    hams = [synthetic.random_molecule(sd).hamiltonian for sd in range(nmol)]
    Ns = [h.wavefunction_data.geminal_data.num_electron_up + h.wavefunction_data.geminal_data.num_electron_dn for h in hams]
    W = [int(np.clip(round(256 + 3840 * (n - 2) / 58), 256, 4096)) for n in Ns]
    mb = MoleculeBatch(hams, W, precision="mixed", seed=11)
    state_gb = sum(gs.walker_bytes("mixed") * w for gs, w in zip(mb.systems, W)) / 1e9
    tuned = mb.autotune(K=4, candidates=(32, 64, 128), reps=1)
    mb.capture(steps, K)
    mb.replay()                                   # warm-up replay
    torch.cuda.synchronize()
    p0 = mb.proposals
    acc0 = sum(int(b.accept.sum()) for b in mb.buckets)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    mb.replay()
    e1.record()
    torch.cuda.synchronize()
    ms_mixed = e0.elapsed_time(e1)
    total = mb.total_walkers
    acc_mixed = (sum(int(b.accept.sum()) for b in mb.buckets) - acc0) / ((mb.proposals - p0) * total)
    buckets = {str(b.bound): {"molecules": len(b.items), "walkers": b.total, "threads": b.threads} for b in mb.buckets}
    launches = mb.graph_launches
    mb.close()
    del mb
    torch.cuda.empty_cache()
    # plain FP64: one launch per molecule, in sequence (each molecule's walkers are
    # built, warmed up, timed and freed in turn; the launch times are summed)
    ms_fp64, acc_fp64 = 0.0, 0
    for k, (h, w) in enumerate(zip(hams, W)):
        sb = MoleculeBatch([h], [w], precision="fp64", seed=11 + k)
        bk = sb.buckets[0]
        idr, fdr = sb.draws(bk, 4)
        sb.sweep(bk, idr, fdr, threads=64)       # warm-up
        idr, fdr = sb.draws(bk, fp64_steps)
        torch.cuda.synchronize()
        a0 = int(bk.accept.sum())
        e0.record()
        sb.sweep(bk, idr, fdr, threads=64)
        e1.record()
        torch.cuda.synchronize()
        ms_fp64 += e0.elapsed_time(e1)
        acc_fp64 += int(bk.accept.sum()) - a0
        sb.close()
        del sb, idr, fdr
    acc_fp64 /= fp64_steps * total
    torch.cuda.empty_cache()
    v_mixed = total * steps / (ms_mixed / 1e3)
    v_fp64 = total * fp64_steps / (ms_fp64 / 1e3)
    return {"workload": f"{nmol} random molecules, {min(Ns)}-{max(Ns)} electrons, {total} walkers (256-4096 per molecule, "
                        f"in proportion to the electron count), VMC",
            "mixed_batched_graph": {"walker_steps_per_s": v_mixed, "proposals_per_walker": steps, "ms": ms_mixed,
                                    "walker_state_GB": state_gb,
                                    "rebuild_every": K, "graph_launches": launches, "accept_ratio": acc_mixed,
                                    "buckets": buckets, "autotune": {str(k): v for k, v in tuned.items()}},
            "fp64_per_molecule_sequential": {"walker_steps_per_s": v_fp64, "proposals_per_walker": fp64_steps, "ms": ms_fp64,
                                             "launches": nmol, "accept_ratio": acc_fp64},
            "speedup": v_mixed / v_fp64,
            "note": "aggregate walker-steps/s; CUDA events around one graph replay (mixed) and around the 64 sequential "
                    "launches (FP64); draws resident in HBM"}


def vmc_leg(walkers: int = 16384, K: int = 32, rounds: int = 3):
    """VMC on the 32-nucleus chain (96 electrons, 736 AOs), the VMC half of the
    precision workload: the mixed form (float tables, warp-parallel float
    proposal, batched sweep of one molecule) with its drift-control rebuild
    after every K proposals, against the same sweep in FP64 from the same
    configurations with the same draws.  Reports walker-steps/s of
    both, the acceptance ratios and the fraction of walkers whose paths agree."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.batching import MoleculeBatch
    syn = synthetic.chain32()
    mb = MoleculeBatch([syn.hamiltonian], [walkers], precision="mixed", seed=5)
    gs = mb.systems[0]
    bk = mb.buckets[0]
    tuned = mb.autotune(K=4, candidates=(64, 128), reps=1)
    mb.rebuild(True)
    start = mb.walkers[0].r.clone()
    draws = [mb.draws(bk, K) for _ in range(rounds + 1)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    mb.sweep(bk, *draws[0])   # warm-up round
    mb.rebuild(False)
    torch.cuda.synchronize()
    a0 = int(bk.accept.sum())
    e0.record()
    for i in range(1, rounds + 1):
        mb.sweep(bk, *draws[i])
        mb.rebuild(False)
    e1.record()
    torch.cuda.synchronize()
    ms_mixed = e0.elapsed_time(e1)
    acc_mixed = (int(bk.accept.sum()) - a0) / (rounds * K * walkers)
    r_mixed = mb.walkers[0].r.clone()
    state_gb = gs.walker_bytes("mixed") * walkers / 1e9
    mb.close()
    del mb
    torch.cuda.empty_cache()
    # plain FP64: the same sweep in FP64 (no energy-cache upkeep either), from the
    # same configurations with the same draws
    sb = MoleculeBatch([syn.hamiltonian], [walkers], precision="fp64", seed=5)
    sk = sb.buckets[0]
    sb.walkers[0].r.copy_(start)
    sb.rebuild(True)
    sb.sweep(sk, *draws[0], threads=64)   # warm-up round
    torch.cuda.synchronize()
    a0 = int(sk.accept.sum())
    e0.record()
    for i in range(1, rounds + 1):
        sb.sweep(sk, *draws[i], threads=64)
    e1.record()
    torch.cuda.synchronize()
    ms_fp64 = e0.elapsed_time(e1)
    acc_fp64 = (int(sk.accept.sum()) - a0) / (rounds * K * walkers)
    same = float(((sb.walkers[0].r - r_mixed).abs().amax(dim=(1, 2)) < 1e-6).double().mean())
    sb.close()
    del sb, draws, start, r_mixed
    torch.cuda.empty_cache()
    v_mixed = walkers * K * rounds / (ms_mixed / 1e3)
    v_fp64 = walkers * K * rounds / (ms_fp64 / 1e3)
    return {"workload": f"VMC chain32, {walkers} walkers, {rounds} x {K} single-electron proposals, step 0.4 bohr",
            "mixed": {"walker_steps_per_s": v_mixed, "ms": ms_mixed, "accept_ratio": acc_mixed, "walker_state_GB": state_gb,
                      "threads": bk.threads, "autotune": {str(k): v for k, v in tuned.items()},
                      "rebuild_every": K},
            "plain_fp64": {"walker_steps_per_s": v_fp64, "ms": ms_fp64, "accept_ratio": acc_fp64},
            "speedup": v_mixed / v_fp64,
            "same_path_fraction": same,
            "note": "CUDA events around the timed rounds; mixed rounds include the FP64-accurate drift-control "
                    "rebuild of the float tables; draws resident in HBM"}


def config0_leg(walkers: int = 1024, K: int = 40, blocks: int = 5):
    """Config 0: plain FP64 VMC on the JSD water-like molecule, 1024 walkers,
    single-electron Metropolis proposals (step 0.4 bohr) with E_L every K = 40
    proposals, through MCMC.run_block (jqmc_mcmc.py:4278-4533, :725-747).
    walker-steps/s counts proposals; the energy's share of the time is reported."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_mcmc import MCMC
    syn = synthetic.water_like()
    m = MCMC(syn.hamiltonian, mcmc_seed=3, num_walkers=walkers, num_mcmc_per_measurement=K, Dt=0.4, epsilon_AS=0.0)
    draws = [m.draws() for _ in range(blocks + 2)]
    for d in draws[:2]:
        m.run_block(*d)
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record()
    for d in draws[2:]:
        m.run_block(*d)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    e0.record()
    for d in draws[2:]:
        m.walkers.vmc_measure(d[2], 0.0)
    e2.record()
    torch.cuda.synchronize()
    ms_e = e0.elapsed_time(e2)
    acc = m.accepted_moves / max(1, m.accepted_moves + m.rejected_moves)
    out = {"workload": f"VMC FP64, JSD water-like (8 electrons, {m.sys.A} AOs), {walkers} walkers, {blocks} x {K} proposals "
                       f"+ E_L per block", "walker_steps_per_s": walkers * K * blocks / (ms / 1e3), "ms": ms,
           "energy_share": ms_e / ms, "accept_ratio": acc,
           "note": "CUDA events around MCMC.run_block (sweep + E_L); draws resident in HBM"}
    del m, draws
    torch.cuda.empty_cache()
    return out


def config1_leg(walkers: int = 8192, K: int = 40, cycles: int = 2):
    """Config 1: plain FP64 LRDMC (GFMC_n) on the 12-nucleus ring (30 electrons,
    JAGP), 8192 walkers, a = 0.2 bohr, 40 projections per branching: the GPU
    drop-in baseline; the mixed form on the same cycle beside it."""
    import torch

    from jqmc_gb300 import synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    syn = synthetic.ring12()
    out = {"workload": f"LRDMC GFMC_n, 12-nucleus ring (30 electrons), {walkers} walkers, {K} projections per branching, "
                       f"a = 0.2 bohr"}
    for form in ("fp64", "mixed"):
        g = GFMC_n(syn.hamiltonian, num_walkers=walkers, num_mcmc_per_measurement=K, mcmc_seed=9, alat=0.2,
                   precision=form)
        draws = [g.draws() for _ in range(cycles + 1)]
        g.run_block(draws[0], 0.5)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for d in draws[1:]:
            g.run_block(d, 0.5)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[form] = {"walker_steps_per_s": walkers * K * cycles / (ms / 1e3), "ms_per_cycle": ms / cycles}
        del g, draws
        torch.cuda.empty_cache()
    out["speedup_mixed_vs_fp64"] = out["mixed"]["walker_steps_per_s"] / out["fp64"]["walker_steps_per_s"]
    out["note"] = "CUDA events around GFMC_n.run_block (projections, rebuild, energy, comb, gather); draws resident in HBM"
    return out


def gpu_arm(a):
    import ctypes

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    # the CPU baseline runs first, in spawned processes, before any CUDA context exists
    cpu_base = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        budget = 12.0
        cores = os.cpu_count() or 1
        v, done = oracle_rate(a.workload, a.alat, cores, budget, a.nproj)
        cpu_base = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                    "sample": f"{cores} single-threaded processes x 1 walker of {a.workload}, {done} walker-steps in "
                              f"branching cycles of {a.nproj} walker-batched NumPy GFMC_n steps and the block energy "
                              f"(oracle/batched.py), whole cycles for at least {budget:.0f} s"}
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from jqmc_gb300 import _lib, synthetic
    from jqmc_gb300.engine import WalkerSet
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    from jqmc_gb300.replicas import max_over_ranks
    from jqmc_gb300.workload import EXP_F32, EXP_FLOPS, lrdmc_step_bytes, lrdmc_step_flops, lrdmc_step_split

    syn = synthetic.SYSTEMS[a.workload]()
    W, K = a.walkers, a.nproj
    r_up, r_dn = syn.initial_electrons(W, seed=1234 + rank)
    stream = torch.cuda.current_stream()
    L = _lib.lib()
    total = a.warmup + a.steps
    forms = {}
    draws_keep = None
    # the plain FP64 comparison arm runs fewer branching cycles (it is ~8x slower)
    plan = {"fp64": (min(a.warmup, 1), max(1, a.steps // 2)), "mixed": (a.warmup, a.steps)}
    for form in ("fp64", "mixed"):
        drv = GFMC_n(syn.hamiltonian, num_walkers=W, num_mcmc_per_measurement=K, mcmc_seed=7 + rank, alat=a.alat,
                     init_r_up=r_up, init_r_dn=r_dn, precision=form)
        dev = drv.sys.device
        if draws_keep is None:
            draws_keep = [drv.draws() for _ in range(total)]
            zetas = [float(x) for x in np.random.default_rng(99 + rank).random(total)]
        clk = ClockSampler(torch.cuda.current_device()) if (rank == 0 and form == "mixed") else None
        if clk:
            time.sleep(0.4)
        fw, fs = plan[form]
        ms, sums, proj, rb = _time_form(drv, draws_keep, zetas, fw, fs, stream, world, dev)
        clocks = clk.stop() if clk else None
        forms[form] = {"drv": drv, "ms": ms, "sums": sums, "proj": proj, "rebuild": rb, "clocks": clocks, "steps": fs, "warmup": fw,
                       "value": W * K * fs * world / (ms / 1e3)}
        if form == "fp64":
            # free the plain form's state before the mixed form allocates its own
            del drv
            forms["fp64"].pop("drv")
            torch.cuda.empty_cache()
    mixed, plain = forms["mixed"], forms["fp64"]
    gs = mixed["drv"].sys
    dev = gs.device

    # accuracy of the mixed form against the FP64 form, in the order of a branching
    # cycle: both forms start from the same sampled configurations, project one full
    # block (K steps) with the same draws (the mixed form's float rank-1 updates
    # drift as in production), rebuild the carried tables in FP64, and evaluate e_L;
    # e_L is compared on the walkers whose paths coincided
    ws_m = mixed["drv"].walkers
    n_cmp = min(W, 1024)
    r = ws_m.r[:n_cmp].cpu().numpy()
    ref = WalkerSet(gs, r[:, : gs.n_up], r[:, gs.n_up:], precision="fp64")
    mix = WalkerSet(gs, r[:, : gs.n_up], r[:, gs.n_up:], precision="mixed")
    blk = draws_keep[0][:n_cmp].contiguous()
    wr = torch.ones(n_cmp, dtype=torch.float64, device=dev)
    wm = torch.ones_like(wr)
    ref.lrdmc_project(blk, a.alat, 0.0, wr)
    mix.lrdmc_project(blk, a.alat, 0.0, wm)
    ref.rebuild()
    mix.rebuild()
    same = ((ref.r - mix.r).abs().amax(dim=(1, 2)) < 1e-6)
    last = draws_keep[-1][:n_cmp, -1].contiguous()
    e64, _ = ref.lrdmc_energy(last, a.alat)
    e32, _ = mix.lrdmc_energy(last, a.alat)
    flagged = (mix.energy_cancellation() > _lib.FAST_ENERGY_CANCEL)[same].cpu().numpy()
    de = (e32 - e64)[same].cpu().numpy()
    relw = ((wm - wr).abs() / wr.abs())[same].cpu().numpy()
    eL_rms = float(np.sqrt(np.mean(de**2)))
    same_frac = float(same.double().mean())
    # the same configurations with the compensated-float block energy (precision
    # "mixed_fast_energy": the same float tables, read through a second descriptor)
    fast = copy.copy(mix)
    fast.precision = "mixed_fast_energy"
    ee, _ = fast.lrdmc_energy(last, a.alat)
    de_e = (ee - e64)[same].cpu().numpy()
    del ref, mix, fast

    # e2e through the public driver API (mixed form): draws from pinned host memory, sums to host
    drv = mixed["drv"]
    host_draws = [d.cpu().pin_memory() for d in draws_keep[: a.steps]]
    dev_buf = torch.empty_like(draws_keep[0])
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    te0 = time.perf_counter()
    for s in range(a.steps):
        dev_buf.copy_(host_draws[s], non_blocking=True)
        out = drv.run_block(dev_buf, zetas[s]).cpu()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - te0, device=dev)
    e2e = {"value": W * K * a.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(host_draws[0].numel() * 8),
           "d2h_bytes_per_step": int(out.numel() * 8)}

    # roofline: the mixed projection kernel (FP32 part against a measured FP32 FMA peak, FP64 part
    # against the measured FP64 peak) and the plain kernel (FP64)
    r_all = ws_m.r.reshape(W, -1, 3)
    pos = torch.as_tensor(gs._keep["pos"], device=dev)
    near = torch.cdist(r_all, pos[None].expand(W, -1, -1)).argmin(-1)
    maxl1 = torch.as_tensor(gs._keep.get("maxl1", np.zeros(len(gs._keep["pos"]), dtype=np.int32)), device=dev)
    ecp_frac = float((maxl1[near] > 0).double().mean())
    peak64 = _probe(L, L.jqmc_probe_fp64, dev, stream, torch.float64)
    peak32 = _probe(L, L.jqmc_probe_fp32, dev, stream, torch.float32)
    f32, f64 = lrdmc_step_split(gs, ecp_frac)
    mix_ms = sum(mixed["proj"]) / len(mixed["proj"])
    plain_ms = sum(plain["proj"]) / len(plain["proj"])
    ach32 = f32 * W * K / (mix_ms / 1e3) / 1e9
    ach64 = f64 * W * K / (mix_ms / 1e3) / 1e9
    plain_flops = lrdmc_step_flops(gs, ecp_frac) * W * K
    plain_ach = plain_flops / (plain_ms / 1e3) / 1e9
    # DRAM bytes (read + write) per walker-step of the mixed projection kernel from
    # one ncu capture of a small chain32 case (912 walkers x 2 projections: 4.63 GB
    # read, 0.70 GB written), scaled to this launch by the walker-steps it
    # processes (the kernel's traffic grows in proportion)
    traffic_per_ws = NCU_TRAFFIC_PER_WALKER_STEP.get(a.workload)
    traffic = traffic_per_ws * W * K if traffic_per_ws else None
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        peaks = {}
    # block-energy launch times of the two variants on the full walker set: the
    # throughput the mixed form reaches with the compensated-float energy
    last_full = draws_keep[-1][:, -1].contiguous()
    fastw = copy.copy(ws_m)
    fastw.precision = "mixed_fast_energy"
    e_ms = {}
    for label, wsx in (("adaptive", ws_m), ("fast", fastw)):
        wsx.lrdmc_energy(last_full, a.alat)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        wsx.lrdmc_energy(last_full, a.alat)
        e1.record(stream)
        torch.cuda.synchronize()
        e_ms[label] = e0.elapsed_time(e1)
    del fastw
    ws_m.lrdmc_energy(last_full, a.alat)   # leaves the bounds of the full walker set in the scratch
    flagged_full = float((ws_m.energy_cancellation() > _lib.FAST_ENERGY_CANCEL).double().mean())
    cycle_ms = mixed["ms"] / a.steps
    fast_value = W * K * world / ((cycle_ms - e_ms["adaptive"] + e_ms["fast"]) / 1e3)
    # the remaining legs run after the chain32 walker sets are released
    del drv, ws_m, r_all, near
    mixed.pop("drv")
    torch.cuda.empty_cache()
    def leg(run, skip):
        """A further leg on rank 0; an exception is recorded in the line instead of ending the run."""
        if rank != 0 or skip:
            return None
        try:
            return run()
        except Exception as ex:
            torch.cuda.empty_cache()
            return {"error": repr(ex)}

    adjoint = leg(lambda: adjoint_leg(stream, dev, peak64, peaks.get("hbm_gbs")), a.no_adjoint)
    forces = leg(lambda: forces_leg(stream), a.no_adjoint)
    batching = leg(batching_leg, a.no_batching)
    vmc = leg(vmc_leg, a.no_vmc)
    config0 = leg(config0_leg, a.no_configs)
    config1 = leg(config1_leg, a.no_configs)
    bytes_launch = lrdmc_step_bytes(gs, 4) * W * K     # float tables
    ach_hbm = bytes_launch / (mix_ms / 1e3) / 1e9
    hbm_peak = peaks.get("hbm_gbs")
    per_call = {"jqmc_lrdmc_project": 1, "jqmc_lrdmc_energy": 2, "jqmc_branch_comb": 2, "jqmc_walker_gather": 10 if gs.A3 else 8,
                "jqmc_lu_rebuild_refine": 2}   # k_rebuild_m + k_walker_init
    if rank == 0:
        line = {
            "metric": METRIC, "value": mixed["value"], "unit": UNIT,
            "accuracy": {"eL_rms_Ha": eL_rms, "dE_mean_Ha": float(np.mean(de)), "eL_max_Ha": float(np.max(np.abs(de))),
                         "configs": int(len(de)), "bar": "eL_rms<=1e-5 Ha, |dE_mean|<=1e-4 Ha"},
            "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": mixed["ms"] / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": f"lrdmc_{a.workload}", "form": "mixed precision (headline) vs plain FP64", "walkers": W,
                       "projections_per_branching": K, "alat": a.alat, "electrons": gs.N, "aos": gs.A, "j3_aos": gs.A3,
                       "nuclei": len(gs._keep["pos"]),
                       "parallelism": "walkers (one CTA per walker)" + ("; replicas" if world > 1 else ""),
                       "l2": f"walker state {gs.walker_bytes('mixed') * W / 2**20:.0f} MiB (mixed) / "
                             f"{gs.walker_bytes('fp64') * W / 2**20:.0f} MiB (fp64) > L2, no flush"},
            "plain_fp64": {"value": plain["value"], "ms_per_step": plain["ms"] / plain["steps"], "dtype": "f64",
                           "steps": plain["steps"], "warmup": plain["warmup"],
                           "phase_ms": {"projection": plain_ms, "rebuild": float(np.mean(plain["rebuild"]))}},
            "phase_ms": {"projection": mix_ms, "rebuild": float(np.mean(mixed["rebuild"])),
                         "rest": mixed["ms"] / a.steps - mix_ms - float(np.mean(mixed["rebuild"])),
                         "note": "per branching cycle, CUDA events on the launching stream; rest = energy, sums, comb, gather"},
            "speedup_vs_plain_fp64": mixed["value"] / plain["value"],
            "block_energy": {"adaptive_ms": e_ms["adaptive"], "fp64_recomputed_fraction": flagged_full,
                             "cancellation_threshold": _lib.FAST_ENERGY_CANCEL,
                             "note": "compensated-float energy; walkers whose mesh ratios cancel strongly (mean "
                                     "cancellation factor above the threshold) recomputed in FP64 arithmetic (second "
                                     "launch, the other CTAs exit at once)"},
            "fast_block_energy_variant": {"value": fast_value, "speedup_vs_plain_fp64": fast_value / plain["value"],
                                          "energy_ms": e_ms["fast"],
                                          "note": "precision mixed_fast_energy: the cycle with the compensated-float "
                                                  "energy alone, no FP64 recompute (accuracy under accuracy.fast_block_energy_variant)"},
            "accuracy_detail": {"eL_rms_Ha": eL_rms, "eL_max_Ha": float(np.max(np.abs(de))), "configs": int(len(de)),
                         "same_path_fraction": same_frac, "block_weight_rel_diff_max": float(np.max(relw)),
                         "dE_mean_Ha": float(np.mean(de)), "dE_mean_stderr_Ha": float(np.std(de) / np.sqrt(len(de))),
                         "fp64_recomputed_fraction": float(flagged.mean()),
                         "fast_block_energy_variant": {"eL_rms_Ha": float(np.sqrt(np.mean(de_e**2))),
                                                       "eL_max_Ha": float(np.max(np.abs(de_e))),
                                                       "eL_max_unflagged_Ha": float(np.max(np.abs(de_e[~flagged]))),
                                                       "eL_max_flagged_Ha": float(np.max(np.abs(de_e[flagged]))) if flagged.any() else 0.0,
                                                       "dE_mean_Ha": float(np.mean(de_e))},
                         "note": "mixed minus FP64 local energy after one K-step projection block from the same sampled "
                                 "configurations with the same draws and the FP64 rebuild of the carried tables (the "
                                 "order of a branching cycle); adaptive block energy (compensated float, FP64 for the "
                                 "walkers whose mesh ratios cancel strongly); dE_mean is the bias the mixed form adds to <E>",
                         "bar": "|dE_L| <= 1e-5 Ha rms per configuration; |d<E>| <= 1e-4 Ha"},
            "e2e": e2e,
            "gpu_launches": sum(per_call.values()) * a.steps,
            "roofline": {"bound": "hbm", "achieved": ach_hbm, "peak": hbm_peak, "unit": "GB/s",
                         "frac": ach_hbm / hbm_peak if hbm_peak else None,
                         "traffic": traffic, "traffic_unit": "bytes per launch (ncu, scaled from 912 walkers x 2 steps)",
                         "kernel": "k_lrdmc<float,float,float> (jqmc_lrdmc_project, mixed)",
                         "algorithmic_bytes_per_launch": bytes_launch, "avg_launch_ms": mix_ms,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                         "bytes_model": "per walker-step: derivative tables of every electron, T rows and J3 field read, "
                                        "rank-1 updates of T and the J3 field read and written, the moved electron's "
                                        "tables and cache row written (jqmc_gb300.workload.lrdmc_step_bytes)",
                         "compute_view": {"achieved": ach32, "peak": peak32, "unit": "GFLOP/s", "frac": ach32 / peak32,
                                          "flop_convention": f"FMA=2, add/mul/div/sqrt=1, float exp={EXP_F32:g} "
                                                             f"(mul + SFU ex2), FP64 exp={EXP_FLOPS:g}",
                                          "peak_source": "measured in this run by jqmc_probe_fp32 (8 independent FMA chains per thread)",
                                          "fp64_part": {"achieved": ach64, "peak": peak64, "frac": ach64 / peak64,
                                                        "peak_source": "jqmc_probe_fp64, this run"}},
                         "ecp_electron_fraction": ecp_frac,
                         "plain_fp64_kernel": {"bound": "fp64", "achieved": plain_ach, "peak": peak64, "frac": plain_ach / peak64,
                                               "avg_launch_ms": plain_ms, "unit": "GFLOP/s"}},
            "adjoint": adjoint,
            "forces": forces,
            "batching": batching,
            "vmc": vmc,
            "config0_vmc_water": config0,
            "config1_lrdmc_ring12": config1,
            "cpu_baseline": cpu_base,
            "clocks": mixed["clocks"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
    else:
        gpu_arm(a)


if __name__ == "__main__":
    main()
