"""The empirical autotuner times the planner's candidate block shapes on the
GPU and returns the fastest; a replica run with the tuned shape is an exact
sweep like any other (running energy equals the recompute)."""
import pytest

pytestmark = pytest.mark.gpu


def test_tune_picks_the_fastest_candidate(native_lib):
    sn = native_lib
    from starrynight_gb300 import autotune
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=2)
    rep = sn.Replica(128, 128, 128, T=150.0, seed=2)
    best, results = autotune.tune(params, rep, max_candidates=3, sweeps=3, warmup=1)
    shapes = [r[0] for r in results]
    assert best in shapes and len(shapes) >= 1
    assert min(r[1] for r in results) == dict(results)[best]
    with sn.Simulation(params, [sn.Replica(128, 128, 128, T=150.0, seed=2, block=best)]) as sim:
        s = sim.schedule(0)
        assert (s["bx"], s["by"], s["bz"]) == best
        sim.init_lattice(0)
        sim.set_recompute(0)
        sim.sweep(3)
        E_run = sim.observables()["E_per_site"][0] * 128 ** 3
        E64 = sim.energy(0, "fp64")
    assert abs(E_run - E64) <= 1e-8 * abs(E64)


def test_tune_table_once_per_size(native_lib):
    sn = native_lib
    from starrynight_gb300 import autotune
    params = sn.ModelParams(cutoff=3, seed=4)
    reps = [sn.Replica(32, 32, 32, T=100.0), sn.Replica(48, 48, 48, T=200.0), sn.Replica(32, 32, 32, T=300.0)]
    tuned = autotune.tune_table(params, reps, max_candidates=2, sweeps=2, warmup=1)
    assert tuned[0].block == tuned[2].block and tuned[1].block is not None
    with sn.Simulation(params, tuned) as sim:
        for i in range(3):
            sim.init_lattice(i)
        acc, rej = sim.sweep(2, counts=True)
    assert acc + rej == 2 * (2 * 32 ** 3 + 48 ** 3)


def test_native_autotuner_and_driver_key(native_lib, tmp_path):
    """sn_gpu_autotune (the C-ABI tuner) returns one of the planner's candidates,
    and the driver's AutoTune key runs with it."""
    import subprocess
    sn = native_lib
    from starrynight_gb300 import autotune
    params = sn.ModelParams(cutoff=3, dipoles=(1.0, 0.0), prevalence=(0.8, 0.2), seed=3)
    rep = sn.Replica(48, 48, 48, T=200.0, seed=3)
    shape, ms = autotune.tune_native(params, rep, max_candidates=3, sweeps=2)
    cands = [(c["bx"], c["by"], c["bz"]) for c in sn.plan_candidates(48, 48, 48, 3, False, 3)]
    assert shape in cands and ms > 0.0
    cfg = ("T: 300\nX = 16\nY = 16\nZ = 16\nDipoles = [1.0, 0.0]\nPrevalence = [0.8, 0.2]\n"
           "DipoleCutOff: 3\nMCEqmSteps: 1\nMCMegaSteps: 2\nMCMoves: 2.0\nAutoTune: 3\n")
    (tmp_path / "starrynight.cfg").write_text(cfg)
    r = subprocess.run([sn.driver_path()], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "AutoTune: block " in r.stderr
    assert len([l for l in r.stdout.splitlines() if not l.startswith("#")]) == 2
