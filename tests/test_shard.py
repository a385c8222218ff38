"""Replica tables over ranks (starrynight_gb300/shard.py): the host Philox
against the published known-answer vectors and the oracle, the partition,
and cross-rank replica exchange over a world_size-2 gloo group on the CPU
(ranks agree with each other and with the one-rank run).  The simulation is
a stand-in with deterministic energies: nothing here needs a GPU."""
import os
import socket

import numpy as np
import pytest

from starrynight_gb300 import shard


def test_philox_known_answers_and_oracle():
    # Random123 kat_vectors, philox4x32 R=10
    assert shard.philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert shard.philox4x32_10((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                         0x6D5451FD)
    assert shard.philox4x32_10((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)) == (
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)
    from oracle import oracle as O
    rng = np.random.default_rng(1)
    for _ in range(50):
        c = [int(v) for v in rng.integers(0, 2 ** 32, 4)]
        k = [int(v) for v in rng.integers(0, 2 ** 32, 2)]
        assert shard.philox4x32_10(c, k) == tuple(int(v) for v in O.philox(c, k))


def test_partition_balanced_and_complete():
    costs = [5, 1, 8, 3, 3, 9, 2, 7, 4, 6]
    for ws in (1, 2, 3, 4, 16):
        parts = shard.partition(costs, ws)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        assert parts == shard.partition(costs, ws)  # deterministic


class FakeSim:
    """Stand-in for Simulation: energies are a deterministic function of the
    replica, its temperature and the sweep count."""

    def __init__(self, params, replicas):
        self.replicas = list(replicas)
        self.T = [float(r.T) for r in self.replicas]
        self.n = 0

    def sweep(self, n):
        self.n += n

    def observables(self):
        e = [-(1.0 / t) * 300.0 + 0.05 * np.sin(0.7 * r.seed + 0.3 * self.n) for r, t in zip(self.replicas, self.T)]
        return {"E_per_site": np.array(e)}

    def set_temperature(self, j, T):
        self.T[j] = float(T)

    def close(self):
        pass


class Rep:
    def __init__(self, L, T, seed):
        self.X = self.Y = self.Z = L
        self.T = T
        self.seed = seed

    @property
    def n_sites(self):
        return self.X * self.Y * self.Z


class Params:
    cutoff = 3
    seed = 0xC0FFEE


def _table():
    rng = np.random.default_rng(3)
    return [Rep(int(L), float(t), 100 + i) for i, (L, t) in
            enumerate(zip(rng.choice([8, 12, 16], 12), np.geomspace(50, 500, 12)))]


def _run(rank, ws, reduce_sum=None):
    sh = shard.ShardedReplicas(Params(), _table(), rank, ws, exchange_every=10, reduce_sum=reduce_sum,
                               simulation_factory=FakeSim)
    sh.sweep(35)
    sh.sweep(25)
    return sh


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=ws)
    try:
        sh = _run(rank, ws)
        local_T = {i: sh.sim.T[j] for j, i in enumerate(sh.local)}
        q.put((rank, [float(t) for t in sh.ladder.T], list(sh.ladder.order), sh.ladder.attempted,
               sh.ladder.accepted, local_T))
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.timeout(120)
def test_exchange_over_two_gloo_ranks_equals_one_rank():
    import torch.multiprocessing as mp
    ref = _run(0, 1)
    assert ref.ladder.attempted == 6 * 6 - 3 and ref.ladder.accepted > 0  # 6 rounds of 6 / 5 pairs
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, T, order, att, acc, local_T in out:
        assert T == [float(t) for t in ref.ladder.T]
        assert order == ref.ladder.order
        assert (att, acc) == (ref.ladder.attempted, ref.ladder.accepted)
        for i, t in local_T.items():  # each rank's simulations run at the ladder's temperatures
            assert t == pytest.approx(float(ref.ladder.T[i]))
    owned = sorted(i for *_, local_T in out for i in local_T)
    assert owned == list(range(len(_table())))
