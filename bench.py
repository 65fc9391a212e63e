"""Walker-path benchmark on GB300: LRDMC (GFMC_n) projections, FP64.

Workload (default): the 12-nucleus synthetic ring -- 6 C-like nuclei (Z_eff 4,
semilocal ECP with l = 0, 1 non-local channels) at 2.64 bohr and 6 H at 4.69
bohr, 30 electrons (15/15), 192 spherical GTOs, JAGP geminal, J1/J2/J3 (60 J3
AOs); 8192 walkers; lattice spacing 0.2 bohr, 6 directions; T-move ECP
(Nv = 6); 40 projections per branching.  One bench step = one branching
cycle: 40 projections of every walker, the local energy, the weighted sums,
the comb reconfiguration and the rebuild of G^-1 / T tables from positions.
walker-steps per bench step = walkers x 40.

value : walker-steps/s with the draws resident in HBM (kernel throughput).
e2e   : the same through the public driver API (jqmc_gb300.jqmc_gfmc.GFMC_n.run_block)
        with the draws copied from pinned host memory each step and the step's
        sums read back to the host.
Walker state is 8192 x 64 KB = 0.5 GB > L2 (129 MB), so no L2 flush is needed.

--impl reference : the CPU oracle (NumPy restatement of the reference, which is
Python/JAX and cannot run without JAX) on all host cores, one process per core,
each projecting its own walker; a bounded sample per step.
"""

from __future__ import annotations

import argparse
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
UNIT = "walker-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="ring12", choices=["ring12", "water_like", "chain32"])
    p.add_argument("--walkers", type=int, default=8192)
    p.add_argument("--nproj", type=int, default=40)
    p.add_argument("--alat", type=float, default=0.2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


# ----------------------------------------------------------------------------- CPU oracle arm
def _oracle_worker(args):
    """Project one walker with the oracle for about `budget` seconds; returns walker-steps done and seconds."""
    workload, seed, alat, budget = args
    from jqmc_gb300 import synthetic
    from oracle import drivers as D
    from oracle.wf import OracleSystem
    syn = synthetic.SYSTEMS[workload]()
    o = OracleSystem(syn.hamiltonian)
    r_up, r_dn = syn.initial_electrons(1, seed=seed)
    st = D.init_state(o, r_up[0], r_dn[0])
    rng = np.random.default_rng(seed)
    w = 1.0
    t0 = time.perf_counter()
    done = 0
    while True:
        draw = np.concatenate([rng.uniform(-2 * np.pi, 2 * np.pi, 3), rng.uniform(size=1)])
        w, _, _, _ = D.lrdmc_step(o, st, w, draw, alat, 0.0)
        done += 1
        if time.perf_counter() - t0 >= budget:
            break
    return done, time.perf_counter() - t0


def oracle_rate(workload: str, alat: float, procs: int, budget: float):
    """walker-steps/s of the oracle with `procs` processes (spawned before any GPU use)."""
    if procs == 1:
        done, secs = _oracle_worker((workload, 0, alat, budget))
        return done / secs, done
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_worker, [(workload, s, alat, budget) for s in range(procs)])
    return sum(d / s for d, s in res), sum(d for d, _ in res)


def reference_arm(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    vals = []
    for _ in range(a.warmup):
        pass
    budget = 15.0
    for _ in range(a.steps):
        v, _ = oracle_rate(a.workload, a.alat, cores, budget)
        vals.append(v)
    v = statistics.median(vals)
    sample = f"{cores} processes x 1 walker of {a.workload}, LRDMC projections for {budget:.0f} s each, {a.steps} samples"
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
def gpu_arm(a):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    # the CPU baseline runs first, in spawned processes, before any CUDA context exists
    cpu_base = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        budget = 12.0
        v, done = oracle_rate(a.workload, a.alat, 1, budget)
        cpu_base = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                    "sample": f"1 walker of {a.workload}, {done} LRDMC projections in {budget:.0f} s (NumPy oracle, 1 process)"}
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from jqmc_gb300 import _lib, synthetic
    from jqmc_gb300.jqmc_gfmc import GFMC_n
    from jqmc_gb300.workload import EXP_FLOPS, lrdmc_step_bytes, lrdmc_step_flops

    syn = synthetic.SYSTEMS[a.workload]()
    W, K = a.walkers, a.nproj
    r_up, r_dn = syn.initial_electrons(W, seed=1234 + rank)
    drv = GFMC_n(syn.hamiltonian, num_walkers=W, num_mcmc_per_measurement=K, mcmc_seed=7 + rank, alat=a.alat,
                 init_r_up=r_up, init_r_dn=r_dn)
    gs = drv.sys
    dev = gs.device
    stream = torch.cuda.current_stream()
    launches = {"n": 0}

    # count our kernel launches: wrap the ctypes entry points used inside a block
    L = _lib.lib()
    per_call = {"jqmc_lrdmc_project": 1, "jqmc_lrdmc_energy": 1, "jqmc_branch_comb": 2, "jqmc_walker_gather": 7 if gs.A3 else 6,
                "jqmc_walker_init": 1}
    # dominant-kernel timing with events on the launching (current) stream
    proj_events = []
    orig_project = drv.walkers.__class__.lrdmc_project

    def timed_project(self, draws, alat, E_scf, w):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        orig_project(self, draws, alat, E_scf, w)
        e1.record(stream)
        proj_events.append((e0, e1))

    total_steps = a.warmup + a.steps
    draws = [drv.draws() for _ in range(total_steps)]
    zetas = [float(x) for x in np.random.default_rng(99 + rank).random(total_steps)]
    for s in range(a.warmup):
        drv.run_block(draws[s], zetas[s])
    torch.cuda.synchronize()

    # ---- timed region: device-resident inputs
    drv.walkers.__class__.lrdmc_project = timed_project
    clk = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    time.sleep(0.4 if clk else 0.0)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    sums = []
    for s in range(a.warmup, total_steps):
        sums.append(drv.run_block(draws[s], zetas[s]))
        launches["n"] += sum(per_call.values())
    t1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = clk.stop() if clk else None
    drv.walkers.__class__.lrdmc_project = orig_project
    from jqmc_gb300.replicas import max_over_ranks
    ms = max_over_ranks(t0.elapsed_time(t1), device=dev)
    walker_steps = W * K * a.steps * world
    value = walker_steps / (ms / 1e3)
    proj_ms = [e0.elapsed_time(e1) for e0, e1 in proj_events]
    proj_avg = sum(proj_ms) / len(proj_ms)
    energies = torch.stack(sums).cpu().numpy()
    e_mean = float(np.mean(energies[:, 2] / energies[:, 1]))

    # ---- e2e: public driver API, draws from pinned host memory, sums back to host
    host_draws = [d.cpu().pin_memory() for d in draws[: a.steps]]
    dev_buf = torch.empty_like(draws[0])
    h2d = host_draws[0].numel() * 8
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    te0 = time.perf_counter()
    for s in range(a.steps):
        dev_buf.copy_(host_draws[s], non_blocking=True)
        out = drv.run_block(dev_buf, zetas[s]).cpu()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - te0, device=dev)
    e2e = {"value": W * K * a.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(out.numel() * 8)}

    # ---- roofline of the dominant kernel (jqmc_lrdmc_project): FP64 pipe
    r_all = drv.walkers.r.reshape(W, -1, 3)
    pos = torch.as_tensor(gs._keep["pos"], device=dev)
    near = torch.cdist(r_all, pos[None].expand(W, -1, -1)).argmin(-1)
    maxl1 = torch.as_tensor(gs._keep.get("maxl1", np.zeros(len(gs._keep["pos"]), dtype=np.int32)), device=dev)
    ecp_frac = float((maxl1[near] > 0).double().mean())
    flops_launch = lrdmc_step_flops(gs, ecp_frac) * W * K
    achieved = flops_launch / (proj_avg / 1e3) / 1e9
    import ctypes
    sink = torch.zeros(1, dtype=torch.float64, device=dev)
    fl = ctypes.c_double()
    pe0 = torch.cuda.Event(enable_timing=True)
    pe1 = torch.cuda.Event(enable_timing=True)
    blocks = torch.cuda.get_device_properties(dev).multi_processor_count * 8
    L.jqmc_probe_fp64(2000, blocks, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(fl), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    pe0.record(stream)
    _lib.check(L.jqmc_probe_fp64(20000, blocks, ctypes.c_void_p(sink.data_ptr()), ctypes.byref(fl),
                                 ctypes.c_void_p(stream.cuda_stream)), "probe")
    pe1.record(stream)
    torch.cuda.synchronize()
    peak = fl.value / (pe0.elapsed_time(pe1) / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "lrdmc_project_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                traffic = json.load(f).get(a.workload)
        except (OSError, ValueError):
            traffic = None
    bytes_launch = lrdmc_step_bytes(gs) * W * K
    if rank == 0:
        peaks = {}
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except (OSError, ValueError):
            peaks = {}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"lrdmc_{a.workload}", "form": "plain FP64", "walkers": W, "projections_per_branching": K,
                       "alat": a.alat, "electrons": gs.N, "aos": gs.A, "j3_aos": gs.A3, "nuclei": len(gs._keep["pos"]),
                       "parallelism": "walkers (one CTA per walker)" + ("; replicas" if world > 1 else ""),
                       "l2": f"walker state {gs.walker_bytes() * W / 2**20:.0f} MiB > L2, no flush"},
            "e2e": e2e,
            "gpu_launches": launches["n"],
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "GFLOP/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel": "k_lrdmc (jqmc_lrdmc_project)",
                         "flop_convention": f"FMA=2, add/mul/div/sqrt=1, FP64 exp={EXP_FLOPS:g}; per launch {flops_launch:.3e} FP64 ops",
                         "peak_source": "measured in this run by jqmc_probe_fp64 (8 independent DFMA chains per thread)",
                         "avg_launch_ms": proj_avg, "ecp_electron_fraction": ecp_frac,
                         "hbm": {"algorithmic_bytes_per_launch": bytes_launch,
                                 "achieved_gbs": bytes_launch / (proj_avg / 1e3) / 1e9, "peak_gbs": peaks.get("hbm_gbs"),
                                 "peak_source": "MEASURED_PEAKS.json"}},
            "cpu_baseline": cpu_base,
            "clocks": clocks,
            "E_mean_Ha": e_mean,
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
