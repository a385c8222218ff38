"""Oracle (c): equilibrium averages of the GPU colour sweep against the
reference's own random-sequential runs.

tests/golden/ref_equilibrium.npz holds per-sweep E/site and |P|/site of the
unmodified reference (MT19937, MC_move, src/starrynight-montecarlo-core.c:
143-191) on a 32^3 lattice, cutoff 3, CageStrain 1, no field, 4 seeds per
temperature, after 300 equilibration sweeps (make_golden.py).  The colour
sweep satisfies detailed balance with the same stationary distribution, so
equilibrium averages -- not trajectories -- must agree within the
seed-to-seed spread of both sides."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_equilibrium.npz")


@pytest.mark.gpu
def test_equilibrium_matches_reference_runs(native_lib):
    sn = native_lib
    d = np.load(GOLD)
    Ts, L, equil, prod = [int(t) for t in d["T"]], int(d["L"]), int(d["equil"]), int(d["prod"])
    nseed = d["E"].shape[1]
    params = sn.ModelParams(cutoff=3, cage_strain=1.0, seed=4242)
    reps = [sn.Replica(L, L, L, T=float(T), seed=1000 * i + k) for i, T in enumerate(Ts) for k in range(nseed)]
    with sn.Simulation(params, reps) as sim:
        for r in range(len(reps)):
            sim.init_lattice(r)
        sim.sweep(equil)
        for r in range(len(reps)):
            sim.history(r)  # drop the equilibration log
        sim.sweep(prod)
        logs = [sim.history(r) for r in range(len(reps))]
    E = np.array([e for e, _ in logs]).reshape(len(Ts), nseed, prod)
    P = np.array([p for _, p in logs]).reshape(len(Ts), nseed, prod)
    for i, T in enumerate(Ts):
        g_seed, r_seed = E[i].mean(axis=1), d["E"][i].mean(axis=1)
        sigma = np.sqrt(g_seed.var(ddof=1) / nseed + r_seed.var(ddof=1) / nseed)
        diff = abs(g_seed.mean() - r_seed.mean())
        assert diff <= 4 * sigma + 2e-3 * abs(r_seed.mean()), (T, g_seed.mean(), r_seed.mean(), sigma)
        gp, rp = P[i].mean(axis=1), d["P"][i].mean(axis=1)
        sp = np.sqrt(gp.var(ddof=1) / nseed + rp.var(ddof=1) / nseed)
        assert abs(gp.mean() - rp.mean()) <= 4 * sp + 2e-3, (T, gp.mean(), rp.mean(), sp)
