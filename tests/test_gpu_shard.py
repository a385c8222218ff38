"""A replica table split over two handles (two ranks' shares, driven in one
process on one GPU) with host-side exchange follows the same temperatures and
gives the same lattices as the whole table in one handle with the device
exchange."""
import numpy as np
import pytest

from starrynight_gb300 import shard

pytestmark = pytest.mark.gpu


def test_two_shards_equal_one_handle(native_lib):
    sn = native_lib
    params = sn.ModelParams(cutoff=3, cage_strain=1.0, seed=0xBEEF)
    Ts = np.geomspace(80.0, 480.0, 8)
    reps = [sn.Replica(L, L, L, T=float(t), efield=(0.0, 0.0, 0.05), seed=300 + i)
            for i, (L, t) in enumerate(zip([16, 24, 16, 32, 24, 16, 32, 24], Ts))]
    every, rounds = 5, 8
    with sn.Simulation(params, reps) as whole:
        for i in range(len(reps)):
            whole.init_lattice(i)
        whole.set_exchange(every)
        whole.sweep(every * rounds)
        T_whole = [whole.temperature(i) for i in range(len(reps))]
        lat_whole = [whole.download(i)[0] for i in range(len(reps))]
        att, acc = whole.exchange_stats()
    parts = [shard.ShardedReplicas(params, reps, rank=r, world_size=2, exchange_every=every) for r in range(2)]
    try:
        for p in parts:
            for j in range(len(p.local)):
                p.sim.init_lattice(j)
        for rnd in range(1, rounds + 1):
            for p in parts:
                p.sim.sweep(every)
            E = sum(p.local_energies() for p in parts)
            for p in parts:
                p.apply_exchange(rnd, E)
        T_sh = [float(t) for t in parts[0].ladder.T]
        lat_sh = {}
        for p in parts:
            for j, i in enumerate(p.local):
                lat_sh[i] = p.sim.download(j)[0]
                assert p.sim.temperature(j) == pytest.approx(T_sh[i])
    finally:
        for p in parts:
            p.close()
    assert acc > 0
    assert (parts[0].ladder.attempted, parts[0].ladder.accepted) == (att, acc)
    np.testing.assert_allclose(T_sh, T_whole, rtol=1e-6)
    for i in range(len(reps)):
        assert np.array_equal(lat_sh[i], lat_whole[i]), i
