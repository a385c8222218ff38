"""GPU tests of the physics around the sweep: random streams, energies
against the FP64 oracle (oracle b), running-total drift, adjoint against the
analytic FP64 gradient and finite differences, the T=0 quench, batching,
replica exchange and error handling."""
import numpy as np
import pytest

from oracle import oracle as O

# Site energies: FP32 local fields against FP64, relative with an absolute
# floor of 1e-5 energy units for |e| < 1 (site energies are O(1..10)).
SITE_REL = 1e-5


def _sim(sn, shape, T=300.0, **kw):
    seed = kw.pop("seed", 11)
    params = sn.ModelParams(seed=seed, **kw)
    return sn.Simulation(params, [sn.Replica(*shape, T=T, seed=seed)])


def _model(shape, p, T=300.0):
    return O.make_model(*shape, p.cutoff, T=T, efield=p.efield, K=p.K, cage_strain=p.cage_strain,
                        constrain_to_x=p.constrain_to_x, dim=p.dim)


@pytest.mark.gpu
def test_device_philox_matches_cpu(native_lib):
    rng = np.random.default_rng(0)
    ctr = rng.integers(0, 2 ** 32, size=(257, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2 ** 32, size=(257, 2), dtype=np.uint64).astype(np.uint32)
    out = native_lib.philox(ctr, key)
    ref = np.stack([O.philox(c, k) for c, k in zip(ctr, key)])
    assert np.array_equal(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("dim,constrain", [(3, False), (2, False), (3, True)])
def test_proposals_bit_exact(native_lib, dim, constrain):
    sn = native_lib
    with _sim(sn, (8, 8, 8), dim=dim, constrain_to_x=constrain, seed=123) as sim:
        sites = np.arange(512, dtype=np.uint32)
        for sweep in (0, 7, 1 << 20):
            out = sim.proposals(0, sites, sweep)
            m = O.make_model(8, 8, 8, 3, dim=dim, constrain_to_x=constrain)
            st = O.make_stream(123, 1.0)
            for i in range(0, 512, 7):
                p, u = O.proposal(m, st, int(i), sweep)
                assert np.array_equal(out[i, :3], p) and out[i, 3] == np.float32(u)


@pytest.mark.gpu
def test_init_lattice_solid_solution(native_lib):
    sn = native_lib
    with _sim(sn, (32, 32, 32), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=3) as sim:
        sim.init_lattice(0)
        xyz, ln = sim.download(0)
    occ = ln > 0
    assert abs(occ.mean() - 0.7) < 0.01
    assert np.all(xyz[~occ] == 0)
    assert np.allclose(np.linalg.norm(xyz[occ], axis=1), 1.0, atol=1e-6)
    assert np.all(np.abs(xyz[occ].mean(axis=0)) < 0.02)  # uniform on the sphere


SITE_CASES = [
    ("config1", (32, 32, 32), dict(cutoff=3)),
    ("vacancy_field", (24, 24, 24), dict(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3))),
    ("rc4_K", (16, 16, 16), dict(cutoff=4, cage_strain=0.5, K=0.4, efield=(0.05, 0.0, 0.05))),
    ("mixture", (16, 16, 16), dict(cutoff=3, dipoles=(1.0, 0.6, 0.0), prevalence=(0.5, 0.3, 0.2))),
    ("slab_rc5", (64, 48, 1), dict(cutoff=5, efield=(0.0, 0.0, 0.3))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,shape,kw", SITE_CASES, ids=[c[0] for c in SITE_CASES])
def test_site_energies_match_fp64(native_lib, name, shape, kw):
    sn = native_lib
    with _sim(sn, shape, **kw) as sim:
        sim.init_lattice(0)
        sim.sweep(3)
        E32, s32 = sim.energy(0, "fp32", site=True)
        E64, s64 = sim.energy(0, "fp64", site=True)
        xyz, ln = sim.download(0)
        run = sim.observables()["E_per_site"][0] * np.prod(shape)
    m = _model(shape, sim.params)
    px, py, pz = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
    ref = O.energy64(m, px, py, pz, ln, site=True)
    occ = ln > 0
    err = np.abs(s32[occ] - ref["site"][occ]) / np.maximum(np.abs(ref["site"][occ]), 1.0)
    assert err.max() <= SITE_REL, err.max()
    # the same errors without the floor: relative where |e| >= 1, and for the
    # sites with |e| < 1 (where the floor makes the bound absolute) their own
    # worst absolute error, which must stay below SITE_REL energy units
    mag = np.abs(ref["site"][occ])
    absx = np.abs(s32[occ] - ref["site"][occ])
    big = mag >= 1.0
    if big.any():
        assert (absx[big] / mag[big]).max() <= SITE_REL
    small = ~big
    print("%s: %.1f %% of occupied sites have |e| < 1; their worst error %.2e (absolute), %.2e (relative)"
          % (name, 100.0 * small.mean(), absx[small].max() if small.any() else 0.0,
             (absx[small] / np.maximum(mag[small], 1e-30)).max() if small.any() else 0.0))
    assert not small.any() or absx[small].max() <= SITE_REL
    assert np.max(np.abs(s64 - ref["site"]) / np.maximum(np.abs(ref["site"]), 1.0)) < 1e-12
    assert abs(E64 - ref["E"]) <= 1e-11 * abs(ref["E"])
    assert abs(E32 - ref["E"]) <= 1e-7 * abs(ref["E"])
    assert abs(run - ref["E"]) <= 1e-7 * abs(ref["E"])  # running FP64 total after 3 sweeps


@pytest.mark.gpu
def test_running_total_has_no_drift(native_lib):
    sn = native_lib
    with _sim(sn, (64, 64, 64), T=150.0, efield=(0, 0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3)) as sim:
        sim.init_lattice(0)
        sim.set_recompute(10, "fp64")
        sim.sweep(100)
        drift, n = sim.drift()
        assert n == 10 and drift < 1e-8
        E_run = sim.observables()["E_per_site"][0] * 64 ** 3
        assert abs(sim.energy(0, "fp64") - E_run) < 1e-8 * abs(E_run)
        e, p = sim.history(0)
        assert len(e) == 100 and np.all(np.isfinite(e)) and np.all(p >= 0)


@pytest.mark.gpu
def test_adjoint_matches_fp64_gradient_and_finite_differences(native_lib):
    """Config-4 parameters on a 20^3 lattice: dE/dp_i against the analytic FP64
    gradient and central FP64 finite differences (h = 1e-4) on 256 random
    sites -- through the oracle's site energy change (the restatement of the
    reference's site_energy, pinned to its golden values), which is exactly
    E(p') - E(p) -- and on 4 sites through the full FP64 total energy, and
    dE/d(Dipole, CageStrain, Efield) against finite differences."""
    sn = native_lib
    shape = (20, 20, 20)
    kw = dict(cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), dipoles=(1.0, 0.0), prevalence=(0.9, 0.1))
    with _sim(sn, shape, **kw) as sim:
        sim.init_lattice(0)
        sim.sweep(5)
        g, dpar, E = sim.adjoint(0)
        xyz, ln = sim.download(0)
    p = sim.params
    m = _model(shape, p)
    px, py, pz = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
    ref = O.energy64(m, px, py, pz, ln, dipole=1.0, grad=True)
    assert abs(E - ref["E"]) <= 1e-7 * abs(ref["E"])
    occ = ln > 0
    scale = np.maximum(np.abs(ref["grad"][occ]), 1.0)
    assert np.max(np.abs(g[occ] - ref["grad"][occ]) / scale) < 1e-5
    assert np.all(g[~occ] == 0)  # a vacancy has no dipole degree of freedom
    assert np.allclose(dpar, ref["dparams"], rtol=1e-6, atol=1e-6)
    rng = np.random.default_rng(7)
    h = 1e-4
    sites = rng.choice(np.nonzero(ln)[0], 256, replace=False)
    # central finite differences of the FP64 total energy; only site i changes, so
    # E(p_i + h e_k) - E(p_i - h e_k) is the difference of the two local FP64 changes
    for i in sites:
        for k in range(3):
            up, dn = xyz[i].copy(), xyz[i].copy()
            up[k] = xyz[i, k] + np.float32(h)
            dn[k] = xyz[i, k] - np.float32(h)
            ep = O.delta_energy64(m, px, py, pz, ln, int(i), up)
            em = O.delta_energy64(m, px, py, pz, ln, int(i), dn)
            fd = (ep - em) / (float(up[k]) - float(dn[k]))
            assert abs(g[i, k] - fd) <= 1e-4 * max(1.0, abs(fd)), (i, k, g[i, k], fd)
    # and a few through the full FP64 energy itself
    for i in sites[:4]:
        for k, arr in enumerate((px, py, pz)):
            o = arr[i]
            arr[i] = o + np.float32(h)
            ep = O.energy64(m, px, py, pz, ln)["E"]
            hp = float(arr[i]) - float(o)
            arr[i] = o - np.float32(h)
            em = O.energy64(m, px, py, pz, ln)["E"]
            hm = float(o) - float(arr[i])
            arr[i] = o
            fd = (ep - em) / (hp + hm)
            assert abs(g[i, k] - fd) <= 1e-4 * max(1.0, abs(fd)), (i, k, g[i, k], fd)
    # parameters: CageStrain, Efield components, Dipole (all occupied lengths)
    def E_of(C=p.cage_strain, Ef=tuple(p.efield), D=1.0):
        mm = O.make_model(*shape, p.cutoff, efield=Ef, K=p.K, cage_strain=C)
        return O.energy64(mm, px, py, pz, (ln * np.float32(D)).astype(np.float32))["E"]
    fd_C = (E_of(C=p.cage_strain + h) - E_of(C=p.cage_strain - h)) / (2 * h)
    assert abs(dpar[1] - fd_C) <= 1e-4 * max(1.0, abs(fd_C))
    for k in range(3):
        up, dn = list(p.efield), list(p.efield)
        up[k] += h
        dn[k] -= h
        fd = (E_of(Ef=tuple(up)) - E_of(Ef=tuple(dn))) / (2 * h)
        assert abs(dpar[2 + k] - fd) <= 1e-4 * max(1.0, abs(fd))
    # lengths are float32: divide by the perturbation actually applied
    Dp, Dm = float(np.float32(1.0 + h)), float(np.float32(1.0 - h))
    fd_D = (E_of(D=1.0 + h) - E_of(D=1.0 - h)) / (Dp - Dm)
    assert abs(dpar[0] - fd_D) <= 1e-4 * max(1.0, abs(fd_D))


@pytest.mark.gpu
def test_quench_descends_on_the_sphere(native_lib):
    sn = native_lib
    shape = (16, 16, 16)
    with _sim(sn, shape, cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), dipoles=(1.0, 0.0),
              prevalence=(0.9, 0.1)) as sim:
        sim.init_lattice(0)
        sim.sweep(10)
        trace = sim.quench(0, 100, 0.02)
        xyz, ln = sim.download(0)
        E_after = sim.observables()["E_per_site"][0] * np.prod(shape)
    assert np.all(np.diff(trace) <= 1e-9 * np.abs(trace[1:]))
    assert trace[-1] < trace[0]
    occ = ln > 0
    assert np.allclose(np.linalg.norm(xyz[occ], axis=1), 1.0, atol=1e-5)
    m = _model(shape, sim.params)
    ref = O.energy64(m, *(np.ascontiguousarray(xyz[:, k]) for k in range(3)), ln)["E"]
    assert abs(trace[-1] - ref) <= 1e-7 * abs(ref) and abs(E_after - ref) <= 1e-7 * abs(ref)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["stencil", "cached"])
def test_batched_replicas_equal_individual_runs(native_lib, method):
    sn = native_lib
    params = sn.ModelParams(cutoff=3, seed=9, sweep_method=method)
    reps = [sn.Replica(32, 32, 32, T=100.0, efield=(0, 0, 0.1), seed=21),
            sn.Replica(48, 48, 48, T=300.0, efield=(0, 0, 0.0), seed=22),
            sn.Replica(24, 16, 24, T=450.0, efield=(0.1, 0, 0), seed=23),
            sn.Replica(40, 40, 1, T=200.0, seed=24)]
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        sim.sweep(5)
        batched = [sim.download(i)[0] for i in range(len(reps))]
        obs = sim.observables()
    for i, r in enumerate(reps):
        with sn.Simulation(params, [r]) as one:
            one.init_lattice(0)
            one.sweep(5)
            assert np.array_equal(one.download(0)[0], batched[i])
            assert abs(one.observables()["E_per_site"][0] - obs["E_per_site"][i]) < 1e-9


@pytest.mark.gpu
def test_replica_exchange_replays_on_cpu(native_lib):
    sn = native_lib
    seed = 0x1234
    Ts = list(np.geomspace(100.0, 400.0, 8))
    params = sn.ModelParams(cutoff=3, seed=seed)
    reps = [sn.Replica(16, 16, 16, T=float(t), seed=100 + i) for i, t in enumerate(Ts)]
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        sim.set_exchange(2)
        order = list(range(8))  # temperature rank -> replica
        cur_T = [np.float32(t) for t in Ts]
        key = [(seed ^ 0x5A5A5A5A) & 0xFFFFFFFF, ((seed >> 32) ^ 0xA5A5A5A5) & 0xFFFFFFFF]
        for s in range(1, 11):
            sim.sweep(1)
            if s % 2:
                continue
            E = sim.observables()["E_per_site"] * 16 ** 3
            rnd = s // 2
            for k in range(rnd & 1, 7, 2):
                a, b = order[k], order[k + 1]
                ba, bb = np.float32(300.0 / np.float64(cur_T[a])), np.float32(300.0 / np.float64(cur_T[b]))
                d = (float(ba) - float(bb)) * (E[a] - E[b])
                u = float(np.float32((int(O.philox([k, rnd, 0, 2], key)[0]) >> 8) * 2.0 ** -24))
                if d >= 0 or u < np.exp(d):
                    cur_T[a], cur_T[b] = cur_T[b], cur_T[a]
                    order[k], order[k + 1] = b, a
            got = [sim.temperature(i) for i in range(8)]
            assert np.allclose(got, [float(t) for t in cur_T], rtol=0, atol=1e-3), (s, got, cur_T)
        att, acc = sim.exchange_stats()
        assert att == 17  # rounds 1..5 alternate 3 odd and 4 even adjacent pairs
        assert sorted(np.round(got, 3)) == sorted(np.round([float(t) for t in np.float32(Ts)], 3))


@pytest.mark.gpu
def test_errors_are_statuses_not_exits(native_lib):
    sn = native_lib
    with pytest.raises(sn.SnError) as e:
        sn.Simulation(sn.ModelParams(cutoff=3), [sn.Replica(25, 25, 25)])
    assert e.value.name == "SN_ERR_SCHEDULE"
    with pytest.raises(sn.SnError) as e:
        sn.Simulation(sn.ModelParams(cutoff=7), [sn.Replica(32, 32, 32)])
    assert e.value.name == "SN_ERR_UNSUPPORTED"
    with _sim(sn, (8, 8, 8), dipoles=(1.0, 0.0), prevalence=(0.5, 0.5)) as sim:
        xyz = np.zeros((512, 3), np.float32)
        xyz[:, 0] = 1
        with pytest.raises(sn.SnError) as e:
            sim.upload(0, xyz, np.full(512, 0.5, np.float32))  # a length the handle does not know
        assert e.value.name == "SN_ERR_ARG"
        with pytest.raises(sn.SnError) as e:
            sim.upload(0, xyz, np.full(512, -1.0, np.float32))  # negative lengths
        assert e.value.name == "SN_ERR_ARG"
        with pytest.raises(sn.SnError):
            sim.set_temperature(3, 100.0)
        sim.upload(0, xyz, np.ones(512, np.float32))  # still usable
        sim.sweep(1)
        out, ln = sim.download(0)
        assert np.all(ln == 1)


@pytest.mark.gpu
def test_mixed_lengths_roundtrip_and_field(native_lib):
    sn = native_lib
    shape = (12, 12, 12)
    with _sim(sn, shape, dipoles=(1.0, 0.5, 0.0), prevalence=(0.4, 0.4, 0.2)) as sim:
        rng = np.random.default_rng(1)
        v = rng.normal(size=(1728, 3)).astype(np.float32)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        ln = rng.choice(np.array([1.0, 0.5, 0.0], np.float32), 1728)
        sim.upload(0, v, ln)
        xyz, l2 = sim.download(0)
        assert np.array_equal(l2, ln) and np.array_equal(xyz[ln > 0], v[ln > 0]) and np.all(xyz[ln == 0] == 0)
        sim.set_field(0, (0.0, 0.0, 0.25))
        m = O.make_model(*shape, 3, efield=(0.0, 0.0, 0.25))
        ref = O.energy64(m, *(np.ascontiguousarray(xyz[:, k]) for k in range(3)), l2)["E"]
        assert abs(sim.observables()["E_per_site"][0] * 1728 - ref) <= 1e-7 * abs(ref)
