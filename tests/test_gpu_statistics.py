"""Oracle (c): equilibrium averages of the GPU colour sweep against the
reference's own random-sequential runs.

tests/golden/ref_equilibrium.npz holds per-sweep E/site and |P|/site of the
unmodified reference (MT19937, MC_move, src/starrynight-montecarlo-core.c:
143-191) on 32^3 lattices, 32 independent seeds per temperature, 200
production sweeps after 500 equilibration sweeps (tests/golden/make_golden.py),
for three Hamiltonians:
  plain     cutoff 3, CageStrain 1, no field, every site occupied,
            T in {500, 700, 1000} K;
  vacfield  cutoff 3, CageStrain 1, 30 % vacancies zeroed after
            solid_solution (src/starrynight-lattice.c:139-171), Efield
            (0, 0, 0.1) (src/starrynight-montecarlo-core.c:120-121), the
            physics of the 256^3 benchmark lattice, T in {300, 500} K;
  rc4cage   cutoff 4, CageStrain 0.5, Efield (0.05, 0, 0.05), 10 % vacancies,
            T in {300, 500} K.
At these temperatures E/site is flat after a few hundred sweeps on both
sides (measured relaxation curves); below them the lattices keep ordering
for thousands to tens of thousands of sweeps (plain at 300 K, vacfield at
150 K, rc4cage at 200 K), which no affordable reference run reaches, and a
comparison there would compare transients of two different dynamics.
The colour sweep satisfies detailed balance with the same stationary
distribution, so equilibrium averages -- not trajectories -- must agree, and
every compared series must be stationary (its second half agrees with its
first half within 3 sigma).

Error bars: each run (one seed) is one block; the runs are independent, so
the standard error of a side's mean is the spread of its run means
(ddof = 1) over sqrt(runs).  The GPU side runs 64 seeds per temperature.
Agreement: |mean_gpu - mean_ref| < 3 sigma_combined, with no added slack."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_equilibrium.npz")
N_SIGMA = 3.0
GPU_SEEDS = 64
CASES = ("plain", "vacfield", "rc4cage")


def _gpu_runs(sn, L, cutoff, cage, efield, occupancy, Ts, equil, prod, salt):
    kw = {} if occupancy >= 1.0 else {"dipoles": (1.0, 0.0), "prevalence": (occupancy, 1.0 - occupancy)}
    params = sn.ModelParams(cutoff=cutoff, cage_strain=cage, efield=efield, seed=4242 + salt, **kw)
    reps = [sn.Replica(L, L, L, T=float(T), seed=100000 * salt + 1000 * i + k)
            for i, T in enumerate(Ts) for k in range(GPU_SEEDS)]
    with sn.Simulation(params, reps) as sim:
        for r in range(len(reps)):
            sim.init_lattice(r)
        sim.sweep(equil)
        for r in range(len(reps)):
            sim.history(r)  # drop the equilibration log
        sim.sweep(prod)
        logs = [sim.history(r) for r in range(len(reps))]
    E = np.array([e for e, _ in logs]).reshape(len(Ts), GPU_SEEDS, prod)
    P = np.array([p for _, p in logs]).reshape(len(Ts), GPU_SEEDS, prod)
    return E, P


def _mean_se(runs):
    """Mean over independent runs and its standard error (one block per run)."""
    m = runs.mean(axis=-1)
    return m.mean(), m.std(ddof=1) / np.sqrt(m.size)


def compare(gpu, ref):
    """(difference, combined sigma) of two sets of runs of one observable."""
    mg, sg = _mean_se(gpu)
    mr, sr = _mean_se(ref)
    return mg - mr, float(np.hypot(sg, sr))


def drift(runs):
    """(second-half mean - first-half mean, its standard error) over independent runs."""
    h = runs.shape[-1] // 2
    dd = runs[..., h:].mean(axis=-1) - runs[..., :h].mean(axis=-1)
    return dd.mean(), dd.std(ddof=1) / np.sqrt(dd.size)


def test_fixture_holds_every_case():
    d = np.load(GOLD)
    assert int(d["seeds"]) >= 16
    for c in CASES:
        E, P, T = d[c + "/E"], d[c + "/P"], d[c + "/T"]
        assert E.shape == P.shape == (len(T), int(d["seeds"]), int(d["prod"]))
        assert np.isfinite(E).all() and np.isfinite(P).all()
        assert d[c + "/equil"].shape == T.shape


def test_reference_runs_are_stationary():
    """The reference's own production series are in equilibrium: no drift of
    E/site between their two halves beyond 3 standard errors."""
    d = np.load(GOLD)
    for c in CASES:
        for i, T in enumerate(d[c + "/T"]):
            m, se = drift(d[c + "/E"][i])
            assert abs(m) < N_SIGMA * se, (c, int(T), m, se)


def test_compare_detects_a_planted_bias():
    """The 3-sigma test on the reference's own runs: two halves of the seeds
    agree, and a bias of 5 standard errors planted in one half is caught."""
    d = np.load(GOLD)
    E = d["plain/E"][0]  # 500 K
    a, b = E[: E.shape[0] // 2], E[E.shape[0] // 2:]
    diff, sig = compare(a, b)
    assert abs(diff) < N_SIGMA * sig
    bias = 5 * sig * (1.0 if diff >= 0 else -1.0)
    diff, sig = compare(a + bias, b)
    assert abs(diff) > N_SIGMA * sig


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_equilibrium_matches_reference_runs(native_lib, case):
    sn = native_lib
    d = np.load(GOLD)
    # the GPU side equilibrates at least as long as the reference did at any
    # of the case's temperatures (all its replicas share one handle)
    equil, prod = int(d[case + "/equil"].max()), int(d["prod"])
    L, cutoff, cage, ex, ey, ez, occ = [float(v) for v in d[case + "/params"]]
    Ts = [int(t) for t in d[case + "/T"]]
    E, P = _gpu_runs(sn, int(L), int(cutoff), cage, (ex, ey, ez), occ, Ts, equil, prod, CASES.index(case))
    bad = []
    for i, T in enumerate(Ts):
        m, se = drift(E[i])
        if not abs(m) < N_SIGMA * se:
            bad.append((T, "GPU E/site not stationary", m, se))
        for name, g, r in (("E/site", E[i], d[case + "/E"][i]), ("|P|/site", P[i], d[case + "/P"][i])):
            diff, sig = compare(g, r)
            if not abs(diff) < N_SIGMA * sig:
                bad.append((T, name, g.mean(), r.mean(), diff, sig))
    assert not bad, bad
