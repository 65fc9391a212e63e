"""Many molecules on one GPU: batched VMC launches, per-bucket tuning, CUDA graphs.

The reference runs one MCMC driver per molecule (jqmc/jqmc_mcmc.py, ``MCMC.run``
:456-1000, vmapped over that molecule's walkers).  Here a set of molecules of
uneven size is grouped into electron-count buckets.  Each bucket is one
``jqmc_batch``: a single launch covers the walkers of every molecule in it, each
CTA taking its molecule's tables.

Per bucket an autotuner picks the CTA size (threads per walker) by timing the
bucket's sweep.  ``capture`` records a whole run into one CUDA graph: sweeps of
K proposals, each followed by the FP64 rebuild of the tables that float rank-1
updates carry (mixed precision), for every bucket.  ``replay`` reruns it with a
single launch from the host.

Draw layout per walker and proposal: idraw (sel in [0, N), up index, dn index,
axis) and fdraw (Gaussian, uniform), as ``MCMC.draws``.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._init_config import initial_electrons
from .engine import GpuSystem, WalkerSet

BUCKET_BOUNDS = (16, 32, 64, 128, 256)   # upper bounds of the electron-count buckets


def bucket_of(n_electrons: int) -> int:
    for b in BUCKET_BOUNDS:
        if n_electrons <= b:
            return b
    raise ValueError(f"{n_electrons} electrons: above the largest bucket")


class _Bucket:
    def __init__(self, bound, items, systems, walkers, device):
        self.bound = bound
        self.items = items
        L = _lib.lib()
        n = len(items)
        sys_arr = (C.c_void_p * n)(*[systems[i].handle for i in items])
        descs = (_lib.Walkers * n)(*[walkers[i].desc() for i in items])
        h = C.c_void_p()
        with torch.cuda.device(device):
            _lib.check(L.jqmc_batch_create(n, sys_arr, descs, C.byref(h)), "jqmc_batch_create")
        self.handle = h
        self.total = int(L.jqmc_batch_walkers(h))
        counts = [walkers[i].nwalk for i in items]
        self.offsets = np.concatenate([[0], np.cumsum(counts)])
        # per-walker draw bounds: (N, n_up, n_dn, 3)
        b = []
        for i, c in zip(items, counts):
            gs = systems[i]
            b.append(np.tile([gs.N, gs.n_up, max(gs.n_dn, 1), 3], (c, 1)))
        self.bounds = torch.as_tensor(np.concatenate(b), dtype=torch.float64, device=device)
        self.accept = torch.zeros(self.total, dtype=torch.int32, device=device)
        self.threads = 64

    def close(self):
        if self.handle:
            _lib.lib().jqmc_batch_destroy(self.handle)
            self.handle = None


class MoleculeBatch:
    """Walkers of many molecules, one precision, grouped into electron-count buckets."""

    def __init__(self, hamiltonians, walkers_per_molecule, precision: str = "mixed", seed: int = 0, Dt: float = 0.4,
                 epsilon_AS: float = 0.0, buckets: bool = True):
        self.precision = precision
        self.Dt, self.epsilon_AS = Dt, epsilon_AS
        self.systems = [GpuSystem(h) for h in hamiltonians]
        self.walkers = []
        for k, (gs, h, W) in enumerate(zip(self.systems, hamiltonians, walkers_per_molecule)):
            st, coul = h.structure_data, h.coulomb_potential_data
            r_up, r_dn = initial_electrons(st.positions, coul.effective_charges, gs.n_up, gs.n_dn, int(W), seed + k)
            self.walkers.append(WalkerSet(gs, r_up, r_dn, precision=precision))
        self.device = self.systems[0].device
        groups = {}
        for i, gs in enumerate(self.systems):
            groups.setdefault(bucket_of(gs.N) if buckets else 0, []).append(i)
        self.buckets = [_Bucket(b, items, self.systems, self.walkers, self.device) for b, items in sorted(groups.items())]
        self.gen = torch.Generator(device=self.device)
        self.gen.manual_seed(seed)
        self.graph = None
        self.proposals = 0

    @property
    def total_walkers(self) -> int:
        return sum(b.total for b in self.buckets)

    def close(self):
        for b in self.buckets:
            b.close()

    # ------------------------------------------------------------------ draws
    def draws(self, bucket: _Bucket, K: int):
        u = torch.rand((bucket.total, K, 4), generator=self.gen, dtype=torch.float64, device=self.device)
        idraw = torch.floor(u * bucket.bounds[:, None, :]).to(torch.int32).contiguous()
        fdraw = torch.stack([torch.randn((bucket.total, K), generator=self.gen, dtype=torch.float64, device=self.device),
                             torch.rand((bucket.total, K), generator=self.gen, dtype=torch.float64, device=self.device)],
                            dim=-1).contiguous()
        return idraw, fdraw

    # ------------------------------------------------------------------ launches
    def sweep(self, bucket: _Bucket, idraw: torch.Tensor, fdraw: torch.Tensor, caches: bool = False, threads: int | None = None):
        K = idraw.shape[1]
        stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        _lib.check(_lib.lib().jqmc_vmc_sweep_batch(bucket.handle, K, C.c_void_p(idraw.data_ptr()), C.c_void_p(fdraw.data_ptr()),
                                                   float(self.Dt), float(self.epsilon_AS), C.c_void_p(bucket.accept.data_ptr()),
                                                   int(threads or bucket.threads), int(caches), stream),
                   "jqmc_vmc_sweep_batch")

    def rebuild(self, full: bool = False):
        stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        for b in self.buckets:
            _lib.check(_lib.lib().jqmc_batch_rebuild(b.handle, int(full), stream), "jqmc_batch_rebuild")

    # ------------------------------------------------------------------ tuning
    def autotune(self, K: int = 8, candidates=(32, 64, 128), reps: int = 2) -> dict:
        """Time each bucket's sweep for each CTA size (these proposals are real
        Metropolis steps, counted in ``proposals``); keep the fastest."""
        chosen = {}
        for b in self.buckets:
            best, best_ms = None, None
            for th in candidates:
                idraw, fdraw = self.draws(b, K)
                self.sweep(b, idraw, fdraw, threads=th)   # first launch at this size
                torch.cuda.synchronize()
                times = []
                for _ in range(reps):
                    idraw, fdraw = self.draws(b, K)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    self.sweep(b, idraw, fdraw, threads=th)
                    e1.record()
                    torch.cuda.synchronize()
                    times.append(e0.elapsed_time(e1))
                ms = min(times)
                if best_ms is None or ms < best_ms:
                    best, best_ms = th, ms
            b.threads = best
            chosen[b.bound] = {"threads": best, "ms_per_proposal": best_ms / K, "molecules": len(b.items), "walkers": b.total}
        self.proposals += K * (1 + reps) * len(candidates)
        return chosen

    # ------------------------------------------------------------------ graphs
    def capture(self, steps: int, K: int, rebuild: bool | None = None):
        """Record ``steps`` proposals per walker (sweeps of K, each followed by the
        table rebuild when ``rebuild``, default: mixed precision) for every bucket
        into one CUDA graph.  The draws are generated now and stay resident."""
        if steps % K:
            raise ValueError("steps must be a multiple of K")
        rebuild = (self.precision != "fp64") if rebuild is None else rebuild
        rounds = steps // K
        self._draws = [[self.draws(b, K) for b in self.buckets] for _ in range(rounds)]
        # run once eagerly at the tuned sizes (sets every kernel's launch attributes)
        for b, (idraw, fdraw) in zip(self.buckets, self._draws[0]):
            self.sweep(b, idraw, fdraw)
        self.proposals += K
        if rebuild:
            self.rebuild(False)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for r in range(rounds):
                for b, (idraw, fdraw) in zip(self.buckets, self._draws[r]):
                    self.sweep(b, idraw, fdraw)
                if rebuild:
                    self.rebuild(False)
        self.graph = g
        self._graph_steps = steps
        per_rebuild = (2 if self.precision != "fp64" else 1) if rebuild else 0   # k_rebuild_m + k_walker_init
        self.graph_launches = rounds * len(self.buckets) * (1 + per_rebuild)
        return g

    def replay(self):
        self.graph.replay()
        self.proposals += self._graph_steps

    def accept_ratio(self) -> float:
        acc = sum(int(b.accept.sum()) for b in self.buckets)
        return acc / max(1, self.proposals * self.total_walkers)
