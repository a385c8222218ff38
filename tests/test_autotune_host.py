"""Host logic of the autotuner (no GPU): one timing per distinct lattice
size, and a cache file that spares the timing of sizes tuned before."""
import json

import starrynight_gb300 as sn
from starrynight_gb300 import autotune


def _fake_tune(calls):
    def tune(params, replica, **kw):
        calls.append((replica.X, replica.Y, replica.Z))
        shape = sn.plan_candidates(replica.X, replica.Y, replica.Z, params.cutoff, False, 1)[0]
        return (shape["bx"], shape["by"], shape["bz"]), [((shape["bx"], shape["by"], shape["bz"]), 1.0)]
    return tune


def test_tune_table_once_per_size_and_cache(tmp_path, monkeypatch, native_lib):
    calls = []
    monkeypatch.setattr(autotune, "tune", _fake_tune(calls))
    params = sn.ModelParams(cutoff=3)
    reps = [sn.Replica(32, 32, 32, T=100.0), sn.Replica(48, 48, 48, T=200.0), sn.Replica(32, 32, 32, T=300.0)]
    cache = str(tmp_path / "tune.json")
    out = autotune.tune_table(params, reps, cache=cache)
    assert calls == [(32, 32, 32), (48, 48, 48)]
    assert out[0].block == out[2].block and out[1].block is not None
    assert [r.T for r in out] == [100.0, 200.0, 300.0]
    saved = json.load(open(cache))
    bid = autotune._build_id()
    assert set(saved) == {bid + "/32x32x32/rc3/uniform/auto", bid + "/48x48x48/rc3/uniform/auto"}
    # a second table: known sizes come from the cache, only the new one is timed
    calls.clear()
    out2 = autotune.tune_table(params, [sn.Replica(48, 48, 48), sn.Replica(64, 64, 64)], cache=cache)
    assert calls == [(64, 64, 64)]
    assert out2[0].block == tuple(saved[bid + "/48x48x48/rc3/uniform/auto"])
    assert len(json.load(open(cache))) == 3
    # another cutoff is another key
    calls.clear()
    autotune.tune_table(sn.ModelParams(cutoff=4), [sn.Replica(48, 48, 48)], cache=cache)
    assert calls == [(48, 48, 48)]
