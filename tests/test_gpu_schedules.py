"""The two sweep schedules -- one dataflow launch per sweep (default) and one
launch per block colour (SN_SCHEDULE=phases) -- make the same moves: every
block reads and writes exactly what the per-colour order gives it, so the
lattices and counters are bit-identical, including replica tables of mixed
shapes, slabs, vacancies and cutoff 5, and whatever grouping of the dataflow
queue is chosen -- for the stencil sweep and for the cached-field sweep."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(sn, monkeypatch, env, params, reps, n=4):
    for k in ("SN_SCHEDULE", "SN_FLOW_GROUP", "SN_SWEEP"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with sn.Simulation(params, reps) as sim:
        for r in range(len(reps)):
            sim.init_lattice(r)
        acc, rej = sim.sweep(n, counts=True)
        stats = sim.flow_stats()
        lat = [sim.download(r)[0] for r in range(len(reps))]
    return acc, rej, lat, stats


def _cases(sn):
    rng = np.random.default_rng(5)
    uneven = [sn.Replica(int(L), int(L), int(L), T=80.0 + 20 * i, seed=40 + i)
              for i, L in enumerate(rng.choice([16, 24, 32, 48], 8))]
    return [
        ("mixture_field", sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.5, 0.0),
                                         prevalence=(0.6, 0.2, 0.2), seed=3), [sn.Replica(48, 32, 64, T=150.0, seed=3)]),
        ("table_3d_2d", sn.ModelParams(cutoff=3, seed=4), uneven + [sn.Replica(96, 64, 1, T=250.0, seed=60)]),
        ("cutoff5", sn.ModelParams(cutoff=5, K=0.3, seed=6), [sn.Replica(48, 48, 48, T=300.0, seed=6)]),
        ("grouped_128", sn.ModelParams(cutoff=3, seed=8), [sn.Replica(128, 128, 128, T=200.0, seed=8)]),
    ]


@pytest.mark.parametrize("method", ["stencil", "cached"])
@pytest.mark.parametrize("idx", range(4))
def test_dataflow_equals_per_colour_launches(native_lib, monkeypatch, idx, method):
    sn = native_lib
    name, params, reps = _cases(sn)[idx]
    a = _run(sn, monkeypatch, {"SN_SCHEDULE": "phases", "SN_SWEEP": method}, params, reps)
    assert a[3]["dataflow"] is False
    for env in ({}, {"SN_FLOW_GROUP": "-1"}, {"SN_FLOW_GROUP": "4"}):
        env = dict(env, SN_SWEEP=method)
        b = _run(sn, monkeypatch, env, params, reps)
        assert b[3]["dataflow"] is True
        assert (a[0], a[1]) == (b[0], b[1]), (name, env)
        for x, y in zip(a[2], b[2]):
            assert np.array_equal(x, y), (name, env)
