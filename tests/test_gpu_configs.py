"""The named workload configurations at their full sizes, checked through
properties that do not need the CPU to redo the whole run:

* 128^3, p = 0.9, cutoff 4, CageStrain 0.5, E = (0.05, 0, 0.05): the adjoint
  dE/dp at 256 random sites of a 300 K snapshot against exact FP64 local
  finite differences (E is linear in one site's dipole), dE/d(parameters)
  against the FP64 recompute, and a 500-step T = 0 quench that never raises
  the energy, keeps unit dipoles and ends at the FP64 recomputed energy.
* 16 x 96^3 at cutoff 5 plus a 2048 x 2048 slab in one handle, T = 300 K,
  E_z swept as a triangle of amplitude 0.3: the polarisation answers the
  field with the sign of the +p.E energy, and every replica's running energy
  stays on its recomputed value.
* 64 replicas of 32..128^3, T log-spaced 50-500 K, E_z in [0, 0.2], cutoff 3,
  exchange every 10 sweeps: temperatures stay a permutation of the ladder,
  exchanges are attempted and accepted, and running energies stay exact.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_adjoint_and_quench_128cubed_cutoff4(native_lib):
    sn = native_lib
    shape = (128, 128, 128)
    kw = dict(cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), dipoles=(1.0, 0.0), prevalence=(0.9, 0.1))
    params = sn.ModelParams(seed=4, **kw)
    with sn.Simulation(params, [sn.Replica(*shape, T=300.0, seed=4)]) as sim:
        sim.init_lattice(0)
        sim.sweep(20)  # the 300 K snapshot
        g, dpar, E = sim.adjoint(0)
        xyz, ln = sim.download(0)
        _, dpar64, _ = sim.adjoint(0, grad=False)
        E64 = sim.energy(0, "fp64")
        trace = sim.quench(0, 500, 0.02)
        xq, lq = sim.download(0)
        Eq64 = sim.energy(0, "fp64")
    assert abs(E - E64) <= 1e-7 * abs(E64)
    m = O.make_model(*shape, 4, efield=kw["efield"], cage_strain=0.5)
    px, py, pz = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
    rng = np.random.default_rng(44)
    sites = rng.choice(np.nonzero(ln)[0], 256, replace=False)
    h = np.float32(1e-3)
    for i in sites:
        p = xyz[i].copy()
        for k in range(3):
            up, dn = p.copy(), p.copy()
            up[k] = p[k] + h
            dn[k] = p[k] - h
            d_up = O.delta_energy64(m, px, py, pz, ln, int(i), up)
            d_dn = O.delta_energy64(m, px, py, pz, ln, int(i), dn)
            fd = (d_up - d_dn) / (float(up[k]) - float(dn[k]))
            assert abs(g[i, k] - fd) <= 1e-4 * max(1.0, abs(fd)), (i, k, g[i, k], fd)
    assert np.all(g[ln == 0] == 0)
    np.testing.assert_allclose(dpar, dpar64, rtol=1e-9, atol=1e-9)
    # quench
    assert np.all(np.diff(trace) <= 1e-9 * np.abs(trace[1:]))
    assert trace[-1] < trace[0]
    occ = lq > 0
    assert np.allclose(np.linalg.norm(xq[occ], axis=1), 1.0, atol=1e-5)
    assert abs(trace[-1] - Eq64) <= 1e-7 * abs(Eq64)


def test_hysteresis_16x96cubed_cutoff5_with_2048_slab(native_lib):
    sn = native_lib
    params = sn.ModelParams(cutoff=5, cage_strain=1.0, seed=5)
    reps = [sn.Replica(96, 96, 96, T=300.0, seed=500 + i) for i in range(16)]
    reps.append(sn.Replica(2048, 2048, 1, T=300.0, seed=600))
    steps, sweeps_per_step, amp = 40, 2, 0.3
    ramp = amp * np.concatenate([np.linspace(0, 1, steps // 4, endpoint=False),
                                 np.linspace(1, -1, steps // 2, endpoint=False),
                                 np.linspace(-1, 0, steps // 4)])
    with sn.Simulation(params, reps) as sim:
        for r in range(len(reps)):
            sim.init_lattice(r)
        sim.set_recompute(0)
        Pz = []
        for ez in ramp:
            for r in range(len(reps)):
                sim.set_field(r, (0.0, 0.0, float(ez)))
            sim.sweep(sweeps_per_step)
            Pz.append(sim.observables()["P_vec"][:, 2] / np.array([r.n_sites for r in reps]))
        Pz = np.array(Pz)
        E_run = sim.observables()["E_per_site"] * np.array([r.n_sites for r in reps])
        E_chk = np.array([sim.energy(r, "fp32") for r in range(len(reps))])
    bulk = Pz[:, :16].mean(axis=1)
    # +p.E: the polarisation points against the field
    assert bulk[ramp > 0.2].mean() < 0 < bulk[ramp < -0.2].mean()
    assert np.corrcoef(ramp, bulk)[0, 1] < -0.5
    assert np.corrcoef(ramp, Pz[:, 16])[0, 1] < -0.5  # the slab too
    assert np.all(np.abs(E_run - E_chk) <= 1e-7 * np.abs(E_chk) + 1e-6)


def test_replica_table_64_uneven_with_exchange(native_lib):
    sn = native_lib
    rng = np.random.default_rng(777)
    sizes = rng.choice([32, 48, 64, 96, 128], size=64)
    T = np.geomspace(50.0, 500.0, 64)
    Ez = rng.uniform(0.0, 0.2, size=64)
    reps = [sn.Replica(int(L), int(L), int(L), T=float(t), efield=(0.0, 0.0, float(e)), seed=777 + i)
            for i, (L, t, e) in enumerate(zip(sizes, T, Ez))]
    params = sn.ModelParams(cutoff=3, cage_strain=1.0, seed=777)
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        sim.set_exchange(10)
        acc, rej = sim.sweep(100, counts=True)
        att, ok = sim.exchange_stats()
        temps = np.array([sim.temperature(i) for i in range(len(reps))])
        E_run = sim.observables()["E_per_site"] * np.array([r.n_sites for r in reps])
        E_chk = np.array([sim.energy(r, "fp32") for r in range(len(reps))])
    assert acc + rej == 100 * sum(r.n_sites for r in reps)  # every site once per sweep
    assert 0 < acc < acc + rej
    assert att == 10 * 32 - 5  # 10 rounds alternating 32 and 31 adjacent pairs
    assert 0 < ok <= att
    np.testing.assert_allclose(np.sort(temps), np.sort(T.astype(np.float32)), rtol=1e-6)
    assert np.all(np.abs(E_run - E_chk) <= 1e-7 * np.abs(E_chk) + 1e-6)


def test_largest_lattice_512cubed(native_lib):
    """512^3 (134 M sites, 2.1 GB): the running energy after two sweeps equals a fresh
    FP32-field recompute and the all-FP64 pass, and every occupied site is attempted once."""
    sn = native_lib
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=51)
    with sn.Simulation(params, [sn.Replica(512, 512, 512, T=150.0, seed=51)]) as sim:
        sim.init_lattice(0)
        sim.set_recompute(0)
        acc, rej = sim.sweep(2, counts=True)
        E_run = sim.observables()["E_per_site"][0] * 512 ** 3
        E32 = sim.energy(0, "fp32")
        E64 = sim.energy(0, "fp64")
        _, ln = sim.download(0)
    occ = int((ln > 0).sum())
    assert acc + rej == 2 * occ
    assert 0 < acc < acc + rej
    assert abs(E_run - E64) <= 1e-8 * abs(E64)
    assert abs(E32 - E64) <= 1e-7 * abs(E64)


def test_oversized_lattices_are_refused(native_lib):
    """More than 2^31 - 1 sites, or a side above 32767, is an argument error before any allocation."""
    sn = native_lib
    params = sn.ModelParams(cutoff=3)
    for shape in ((1300, 1300, 1300), (32768, 2, 2)):
        with pytest.raises(sn.SnError):
            sn.Simulation(params, [sn.Replica(*shape)])
