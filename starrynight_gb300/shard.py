"""Replica tables spread over ranks (one GPU per rank).

Replicas are independent lattices, so N GPUs hold disjoint parts of the
replica table and sweep them with no data exchange.  The only coupling is
replica exchange, which needs every replica's total energy and swaps
temperatures, never lattices: every ``every`` sweeps the ranks sum a vector of
n_rep energies (one all-reduce of doubles) and each rank applies, to its own
replicas, the swaps that all ranks compute identically.

The exchange rule is the device's (``sweep_end_kernel`` in
csrc/sn_kernels.cu): replicas ordered by temperature (stable), round r pairs
ranks k, k+1 for k = r mod 2, r mod 2 + 2, ...; a pair swaps temperatures
when d = (beta_a - beta_b)(E_a - E_b) >= 0 or u < exp(d), with beta the float
300/T and u the 24-bit uniform of Philox4x32-10 at counter (k, r, 0, 2) under
the exchange key derived from the seed.  A table sharded over N ranks
therefore follows the same temperature history as the same table in one
handle (up to exp() rounding at the acceptance boundary).
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

_M0, _M1 = 0xD2511F53, 0xCD9E8D57
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


def philox4x32_10(ctr: Sequence[int], key: Sequence[int]) -> tuple:
    """Philox4x32 with 10 rounds (Salmon et al., SC'11), host restatement of the device generator."""
    c0, c1, c2, c3 = (int(v) & _MASK for v in ctr)
    k0, k1 = (int(v) & _MASK for v in key)
    for r in range(10):
        if r:
            k0 = (k0 + _W0) & _MASK
            k1 = (k1 + _W1) & _MASK
        p0 = _M0 * c0
        p1 = _M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & _MASK, p1 & _MASK, ((p0 >> 32) ^ c3 ^ k1) & _MASK, p0 & _MASK
    return c0, c1, c2, c3


def uniform24(x: int) -> float:
    """Top 24 bits of a 32-bit draw as a float in [0, 1)."""
    return float((int(x) >> 8) * 2.0 ** -24)


def exchange_key(seed: int) -> tuple:
    """The exchange stream's Philox key for a handle seed (as sn_gpu_init derives it)."""
    return (seed ^ 0x5A5A5A5A) & _MASK, ((seed >> 32) ^ 0xA5A5A5A5) & _MASK


def partition(costs: Sequence[float], world_size: int) -> list:
    """Deterministic longest-processing-time partition of replica indices over ranks."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = [0.0] * world_size
    parts = [[] for _ in range(world_size)]
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world_size), key=lambda r: (load[r], r))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


class ExchangeLadder:
    """Host copy of the temperature ladder and the device exchange rule."""

    def __init__(self, temperatures: Sequence[float], seed: int):
        self.T = [np.float32(t) for t in temperatures]
        self.order = sorted(range(len(self.T)), key=lambda i: (float(self.T[i]), i))
        self.key = exchange_key(seed)
        self.attempted = 0
        self.accepted = 0

    @staticmethod
    def beta(T: np.float32) -> float:
        return float(np.float32(300.0 / np.float64(T)))

    def round(self, rnd: int, E_total: Sequence[float]) -> list:
        """One exchange round on the total energies; returns the swapped replica pairs."""
        swaps = []
        n = len(self.T)
        for k in range(rnd & 1, n - 1, 2):
            a, b = self.order[k], self.order[k + 1]
            d = (self.beta(self.T[a]) - self.beta(self.T[b])) * (float(E_total[a]) - float(E_total[b]))
            u = uniform24(philox4x32_10((k, rnd, 0, 2), self.key)[0])
            self.attempted += 1
            if d >= 0.0 or u < np.exp(d):
                self.T[a], self.T[b] = self.T[b], self.T[a]
                self.order[k], self.order[k + 1] = b, a
                self.accepted += 1
                swaps.append((a, b))
        return swaps


def _default_sum(vec: np.ndarray) -> np.ndarray:
    try:
        import torch.distributed as dist
    except ImportError:  # pragma: no cover
        return vec
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vec
    import torch
    backend = dist.get_backend()
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.from_numpy(vec).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()


class ShardedReplicas:
    """This rank's share of a replica table, with cross-rank replica exchange.

    ``params``/``replicas`` describe the whole table; ``rank``/``world_size``
    pick this rank's replicas by :func:`partition` of n_sites x neighbours.
    ``reduce_sum`` sums a float64 vector over ranks (default: a
    torch.distributed all-reduce when a process group is up, else identity).
    """

    def __init__(self, params, replicas: Sequence, rank: int = 0, world_size: int = 1, exchange_every: int = 0,
                 reduce_sum: Callable[[np.ndarray], np.ndarray] | None = None, simulation_factory=None):
        from . import sim as _sim
        self.replicas = list(replicas)
        nb = [_sim.neighbour_count(params.cutoff, r.Z) for r in self.replicas]
        self.parts = partition([r.n_sites * n for r, n in zip(self.replicas, nb)], world_size)
        self.local = self.parts[rank]
        self.every = int(exchange_every)
        self.ladder = ExchangeLadder([r.T for r in self.replicas], params.seed)
        self.reduce_sum = reduce_sum or _default_sum
        factory = simulation_factory or _sim.Simulation
        self.sim = factory(params, [self.replicas[i] for i in self.local]) if self.local else None
        self.sweeps = 0

    def close(self):
        if self.sim is not None:
            self.sim.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def local_energies(self) -> np.ndarray:
        """Total energies of this rank's replicas placed in a table-sized vector (zeros elsewhere)."""
        out = np.zeros(len(self.replicas))
        if self.sim is not None:
            e = self.sim.observables()["E_per_site"]
            for j, i in enumerate(self.local):
                out[i] = e[j] * self.replicas[i].n_sites
        return out

    def apply_exchange(self, rnd: int, E_total: np.ndarray) -> list:
        swaps = self.ladder.round(rnd, E_total)
        if self.sim is not None:
            where = {i: j for j, i in enumerate(self.local)}
            for a, b in swaps:
                for i in (a, b):
                    if i in where:
                        self.sim.set_temperature(where[i], float(self.ladder.T[i]))
        return swaps

    def sweep(self, n: int) -> None:
        """n sweeps of this rank's replicas, exchanging at every multiple of ``every``."""
        done = 0
        while done < n:
            step = n - done
            if self.every > 0:
                step = min(step, self.every - self.sweeps % self.every)
            if self.sim is not None:
                self.sim.sweep(step)
            self.sweeps += step
            done += step
            if self.every > 0 and self.sweeps % self.every == 0 and len(self.replicas) > 1:
                E = self.reduce_sum(self.local_energies())
                self.apply_exchange(self.sweeps // self.every, E)
