"""The cached-field sweep (SN_SWEEP_CACHED): every site's local field kept in
HBM as exact fixed-point sums and updated by accepted moves.

Invariants checked here:
  * the cache after any number of sweeps equals, bit for bit, a fresh field
    pass over the current lattice (sn_gpu_field_cache_check), for uniform and
    mixed lengths, vacancies, K and fields, and after every operation that
    changes dipoles outside the sweep (upload, initialisation, quench);
  * the trajectory does not depend on how it is cut into calls or handles:
    a run resumed from a downloaded lattice in a fresh handle is the run that
    never stopped, bit for bit (the cache is a function of the lattice);
  * the two sweep methods sample the same physics: the running energy of the
    cached sweep matches an FP64 recompute, and its equilibrium E/site agrees
    with the stencil sweep's;
  * what the method cannot take is refused with a clear status.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(sn, **kw):
    kw.setdefault("sweep_method", "cached")
    return sn.ModelParams(**kw)


@pytest.mark.parametrize("kw", [
    dict(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3)),
    dict(cutoff=4, cage_strain=0.5, K=0.4, efield=(0.05, 0.0, 0.05)),
    dict(cutoff=3, dipoles=(1.0, 0.6, 0.0), prevalence=(0.5, 0.3, 0.2), efield=(0.0, 0.1, 0.0)),
    dict(cutoff=5, efield=(0.0, 0.0, 0.3)),
], ids=["vacancy_field", "rc4_K", "mixture", "rc5"])
def test_cache_stays_exact(native_lib, kw):
    sn = native_lib
    shape = (48, 48, 48) if kw["cutoff"] == 5 else (32, 32, 32)
    with sn.Simulation(_params(sn, seed=7, **kw), [sn.Replica(*shape, T=250.0, seed=7)]) as sim:
        assert sim.schedule(0)["field_cache"] == 1
        sim.init_lattice(0)
        assert sim.field_cache_check(0) == 0
        for n in (1, 5, 20):
            sim.sweep(n)
            assert sim.field_cache_check(0) == 0, n
        # changes outside the sweep rebuild the cache
        xyz, ln = sim.download(0)
        rng = np.random.default_rng(1)
        v = rng.normal(size=xyz.shape).astype(np.float32)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        v[ln == 0] = 0.0
        sim.upload(0, v, ln)
        assert sim.field_cache_check(0) == 0
        sim.sweep(3)
        sim.quench(0, 3, 0.05)
        assert sim.field_cache_check(0) == 0
        sim.sweep(3)
        assert sim.field_cache_check(0) == 0


def test_resume_in_a_fresh_handle_is_bit_exact(native_lib):
    sn = native_lib
    params = _params(sn, cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=21)
    rep = sn.Replica(32, 32, 32, T=150.0, seed=21)
    with sn.Simulation(params, [rep]) as a:
        a.init_lattice(0)
        a.sweep(7)
        mid, ln = a.download(0)
        a.sweep(9)
        want, _ = a.download(0)
    with sn.Simulation(params, [rep]) as b:
        b.upload(0, mid, ln)
        b.set_sweep_count(7)
        b.sweep(9)
        got, _ = b.download(0)
    assert np.array_equal(got, want)


def test_running_energy_matches_fp64(native_lib):
    sn = native_lib
    params = _params(sn, cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=5)
    with sn.Simulation(params, [sn.Replica(64, 64, 64, T=150.0, seed=5)]) as sim:
        sim.init_lattice(0)
        sim.set_recompute(10, "fp64")
        sim.sweep(60)
        drift, n = sim.drift()
        assert n == 6 and drift < 1e-8, drift
        E_run = sim.observables()["E_per_site"][0] * 64 ** 3
        assert abs(sim.energy(0, "fp64") - E_run) < 1e-8 * abs(E_run)


def test_methods_sample_the_same_equilibrium(native_lib):
    """16 replicas per method at 300 K, 32^3 with vacancies and a field:
    mean E/site over 100 sweeps after 200 agree within 3 standard errors of
    the replica means."""
    sn = native_lib
    means = {}
    for method in ("stencil", "cached"):
        params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3),
                                seed=99, sweep_method=method)
        reps = [sn.Replica(32, 32, 32, T=300.0, seed=500 + k + (0 if method == "stencil" else 1000))
                for k in range(16)]
        with sn.Simulation(params, reps) as sim:
            assert sim.schedule(0)["field_cache"] == (method == "cached")
            for r in range(len(reps)):
                sim.init_lattice(r)
            sim.sweep(200)
            for r in range(len(reps)):
                sim.history(r)
            sim.sweep(100)
            means[method] = np.array([sim.history(r)[0].mean() for r in range(len(reps))])
    a, b = means["stencil"], means["cached"]
    sig = np.hypot(a.std(ddof=1), b.std(ddof=1)) / np.sqrt(len(a))
    assert abs(a.mean() - b.mean()) < 3 * sig, (a.mean(), b.mean(), sig)


def test_refusals(native_lib):
    sn = native_lib
    from starrynight_gb300._abi import SnError
    # Z not a multiple of 4: no cached schedule; forced -> refused, auto -> stencil
    with pytest.raises(SnError):
        sn.Simulation(_params(sn, cutoff=3, seed=1), [sn.Replica(32, 32, 30, T=300.0)])
    with sn.Simulation(sn.ModelParams(cutoff=3, seed=1), [sn.Replica(32, 32, 30, T=300.0)]) as sim:
        assert sim.schedule(0)["field_cache"] == 0
    # dipoles longer than unit length do not fit the cache's fixed-point range
    with sn.Simulation(_params(sn, cutoff=3, seed=2), [sn.Replica(16, 16, 16, T=300.0)]) as sim:
        xyz = np.zeros((16 ** 3, 3), np.float32)
        xyz[:, 2] = 1.5
        with pytest.raises(SnError):
            sim.upload(0, xyz)
        xyz[:, 2] = 1.0
        sim.upload(0, xyz)
        sim.sweep(2)
        assert sim.field_cache_check(0) == 0


@pytest.mark.parametrize("kw", [dict(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3)),
                                dict(cutoff=3, dipoles=(1.0, 0.6, 0.0), prevalence=(0.5, 0.3, 0.2)),
                                dict(cutoff=5, K=0.2)], ids=["vacancy_field", "mixture", "rc5"])
def test_tma_bulk_tile_load_equals_async_copies(native_lib, monkeypatch, kw):
    """The tile load by TMA bulk row copies on an mbarrier (SN_TILE_COPY=bulk)
    moves the same bytes as the 16-byte cp.async path: identical lattices,
    counters and caches, for both sweep schedules."""
    sn = native_lib
    shape = (48, 48, 48) if kw["cutoff"] == 5 else (32, 48, 32)
    reps = [sn.Replica(*shape, T=200.0, seed=3), sn.Replica(*shape, T=400.0, seed=4)]
    out = {}
    for copy in ("async", "bulk"):
        for sched in ("flow", "phases"):
            monkeypatch.setenv("SN_TILE_COPY", copy)
            monkeypatch.setenv("SN_SCHEDULE", sched)
            with sn.Simulation(_params(sn, seed=11, **kw), reps) as sim:
                for r in range(len(reps)):
                    sim.init_lattice(r)
                acc = sim.sweep(6, counts=True)
                assert all(sim.field_cache_check(r) == 0 for r in range(len(reps)))
                out[copy, sched] = (acc, [sim.download(r)[0] for r in range(len(reps))])
    ref = out["async", "flow"]
    for k, v in out.items():
        assert v[0] == ref[0], k
        assert all(np.array_equal(a, b) for a, b in zip(v[1], ref[1])), k
