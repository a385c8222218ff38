"""Generate the golden fixtures in this directory from the UNMODIFIED
reference sources (driven through ``oracle/_ref/libref_harness.so``, built by
``make -C oracle ref`` where the reference tree is present).

The reference ships no tests, golden vectors or fixtures, so these outputs of
the reference itself are what pin the CPU oracle:

  ref_neighbours.npz    gen_neighbour tables, cutoffs 1..6, 3D and Z == 1
  ref_trajectories.npz  initial lattice (initialise_lattice_random +
                        solid_solution) and the lattice after N MC_move calls,
                        with ACCEPT/REJECT, for several parameter sets
  ref_site_energy.npz   site_energy() values for random trial moves
  ref_equilibrium.npz   per-sweep E/site and |P|/site of random-sequential runs
                        (statistical oracle), 32 seeds per temperature, 32^3:
                        cutoff 3 / CageStrain 1 / no field / all occupied at
                        T in {500,700,1000}; cutoff 3 / 30 % vacancies /
                        Efield (0,0,0.1) at T in {300,500}; cutoff 4 /
                        CageStrain 0.5 / Efield (0.05,0,0.05) / 10 % vacancies
                        at T in {300,500}; 200 production sweeps after a
                        per-temperature equilibration
  ref_analysis.npz      dipole_potential, dipole_electricfield(4),
                        dipole_electricfieldoffset(2) maps, polarisation(),
                        landau_order() and the radial_order_parameter file for
                        random, patterned, slab and mixed lattices
  ref_files.npz         the bytes of every analysis writer on one 10^3 lattice
                        with vacancies, plus the captured stderr of
                        outputlattice_dumb_terminal and recombination_calculator
  ref_driver_files.npz  the files the stock reference binary writes for a 10x12x14
                        "spectrum" run with every analysis flag on and no moves

Usage:  python tests/golden/make_golden.py [--skip-equilibrium] [--analysis-only]
                                          [--equilibrium-only [case ...]]
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

TRAJ_CASES = [
    dict(name="cube8", X=8, Y=8, Z=8, cutoff=3, T=300, moves=20000),
    dict(name="field_K", X=6, Y=8, Z=10, cutoff=2, T=150, efield=(0.1, -0.2, 0.3), K=0.5, cage_strain=0.7,
         moves=20000),
    dict(name="slab", X=12, Y=12, Z=1, cutoff=3, T=300, moves=20000),
    dict(name="constrain_x", X=8, Y=8, Z=8, cutoff=3, T=300, constrain_to_x=True, moves=20000),
    dict(name="vacancies", X=8, Y=8, Z=8, cutoff=3, T=200, lengths=(1.0, 0.0), prevalence=(0.7, 0.3),
         moves=20000),
    dict(name="mixture_rc4", X=10, Y=10, Z=10, cutoff=4, T=250, lengths=(1.0, 0.5, 0.0),
         prevalence=(0.5, 0.3, 0.2), efield=(0.0, 0.0, 0.2), moves=8000),
]

# Statistical oracle: three Hamiltonians, 32 independent reference runs per
# temperature.  "plain" is the small cubic case (all sites occupied, no field);
# "vacfield" the solid solution with vacancies zeroed after solid_solution and
# a field along z (the physics of the 256^3 benchmark lattice); "rc4cage"
# cutoff 4 with a weaker cage strain, an oblique field and 10 % vacancies.
# Temperatures and equilibration lengths come from relaxation curves measured
# on both sides (reference runs on the CPU, 32 GPU replicas up to 20000
# sweeps): at these temperatures E/site is flat after a few hundred sweeps,
# except for cutoff 4 at 300 K, where the reference's random-sequential
# moves still lower E/site by a few 10^-3 between 500 and 1500 sweeps (the
# colour sweep is flat from about 1000): its runs equilibrate for 3000.
# Below these temperatures the lattices keep ordering for thousands (plain
# lattice at 300 K, vacancy lattice at 150 K: still falling after 20000
# sweeps on the GPU) or tens of thousands of sweeps (cutoff 4 at 200 K),
# which no affordable reference run reaches.  The test checks that every
# series it compares is stationary.
EQ_CASES = [
    dict(name="plain", L=32, cutoff=3, cage_strain=1.0, efield=(0.0, 0.0, 0.0), occupancy=1.0, T=(500, 700, 1000),
         equil=(500, 500, 500)),
    dict(name="vacfield", L=32, cutoff=3, cage_strain=1.0, efield=(0.0, 0.0, 0.1), occupancy=0.7, T=(300, 500),
         equil=(500, 500)),
    dict(name="rc4cage", L=32, cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), occupancy=0.9, T=(300, 500),
         equil=(3000, 500)),
]
EQ_SEEDS = 32
EQ_PROD = 200


def _sim(R, c, seed=None):
    return R.RefSim(c["X"], c["Y"], c["Z"], cutoff=c["cutoff"], cage_strain=c.get("cage_strain", 1.0),
                    K=c.get("K", 0.0), efield=c.get("efield", (0.0, 0.0, 0.0)),
                    constrain_to_x=c.get("constrain_to_x", False), T=c["T"],
                    lengths=c.get("lengths", (1.0,)), prevalence=c.get("prevalence", (1.0,)), seed=seed)


def neighbours(R):
    out = {}
    for rc in range(1, 7):
        for Z in (8 * rc + 1, 1):
            s = R.RefSim(4, 4, Z, cutoff=rc)
            dxyz, d = s.neighbours()
            tag = "rc%d_%s" % (rc, "2d" if Z == 1 else "3d")
            out[tag + "_dxyz"] = dxyz
            out[tag + "_d"] = d
    np.savez_compressed(os.path.join(HERE, "ref_neighbours.npz"), **out)


def trajectories(R):
    out = {}
    for c in TRAJ_CASES:
        s = _sim(R, c)
        out[c["name"] + "_init"] = s.lattice()
        s.mc_moves(c["moves"])
        out[c["name"] + "_final"] = s.lattice()
        out[c["name"] + "_counts"] = np.array(s.counts(), np.uint64)
        out[c["name"] + "_beta"] = np.array(s.beta())
    np.savez_compressed(os.path.join(HERE, "ref_trajectories.npz"), **out)


def site_energies(R):
    c = dict(X=8, Y=8, Z=8, cutoff=3, T=300, efield=(0.05, 0.1, -0.2), K=0.4, cage_strain=1.3)
    s = _sim(R, c)
    s.mc_moves(5000)
    lat = s.lattice()
    rng = np.random.default_rng(2024)
    n = 300
    xyz = rng.integers(0, 8, size=(n, 3)).astype(np.int32)
    v = rng.normal(size=(n, 3))
    v = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    dE = np.array([s.site_energy(int(a), int(b), int(cc), v[i]) for i, (a, b, cc) in enumerate(xyz)])
    np.savez_compressed(os.path.join(HERE, "ref_site_energy.npz"), lattice=lat, sites=xyz, new=v, dE=dE,
                        params=np.array([8, 8, 8, 3, 300, 0.05, 0.1, -0.2, 0.4, 1.3]))


def _eq_run(args):
    ci, T, k = args
    from oracle import oracle as O
    from oracle import ref_harness as R
    c = EQ_CASES[ci]
    L = c["L"]
    p = c["occupancy"]
    lengths, prev = ((1.0,), (1.0,)) if p >= 1.0 else ((1.0, 0.0), (p, 1.0 - p))
    # The reference's random_sphere_point tests x1*x1 + x2*x2 > 1 but takes
    # sqrt(1 - x1*x1 - x2*x2), rounded differently: when the sum is within
    # rounding of 1 the square root is of a negative number and the dipole is
    # NaN (src/starrynight-config.c:209-225).  A NaN site never moves and
    # freezes its neighbours, so such an initial lattice is redrawn with the
    # next seed.  (Proposals with NaN are always rejected and never enter
    # the lattice.)
    for attempt in range(100):
        seed = (0xDEADBEEF + T + 7919 * k + 104729 * ci + 15485863 * attempt) & 0xFFFFFFFF
        s = R.RefSim(L, L, L, cutoff=c["cutoff"], cage_strain=c["cage_strain"], efield=c["efield"], T=T,
                     lengths=lengths, prevalence=prev, seed=seed)
        if np.isfinite(s.lattice()).all():
            break
    if p < 1.0:  # vacancies as zero vectors, as on the GPU (src/starrynight-lattice.c:139-171 sets only length)
        lat = s.lattice()
        lat[lat[:, 3] == 0, :3] = 0.0
        s.set_lattice(lat)
    N = L ** 3
    s.mc_moves(c["equil"][c["T"].index(T)] * N)
    m = O.make_model(L, L, L, c["cutoff"], T=T, efield=c["efield"], cage_strain=c["cage_strain"])
    E, P = [], []
    for _ in range(EQ_PROD):
        s.mc_moves(N)
        lat = s.lattice()
        px, py, pz, ln = O.soa(lat)
        E.append(O.energy64(m, px, py, pz, ln)["E"] / N)
        P.append(np.linalg.norm((lat[:, :3].astype(np.float64) * lat[:, 3:4]).sum(axis=0)) / N)
    return ci, T, k, np.array(E), np.array(P)


def equilibrium(only=None):
    """only: names of the cases to run again; the others are kept from the existing file."""
    keep = {}
    path = os.path.join(HERE, "ref_equilibrium.npz")
    if only and os.path.exists(path):
        with np.load(path) as old:
            keep = {k: old[k] for k in old.files}
    jobs = [(ci, T, k) for ci, c in enumerate(EQ_CASES) for T in c["T"] for k in range(EQ_SEEDS)
            if not only or c["name"] in only]
    # longest runs first
    jobs.sort(key=lambda j: -EQ_CASES[j[0]]["cutoff"] * EQ_CASES[j[0]]["equil"][EQ_CASES[j[0]]["T"].index(j[1])])
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(jobs), os.cpu_count() or 4)) as pool:
        res = pool.map(_eq_run, jobs, chunksize=1)
    out = dict(keep)
    out.update({"seeds": EQ_SEEDS, "prod": EQ_PROD})
    for ci, c in enumerate(EQ_CASES):
        if only and c["name"] not in only:
            continue
        E = np.zeros((len(c["T"]), EQ_SEEDS, EQ_PROD))
        P = np.zeros_like(E)
        for cj, T, k, e, p in res:
            if cj == ci:
                i = c["T"].index(T)
                E[i, k], P[i, k] = e, p
        n = c["name"]
        out[n + "/E"], out[n + "/P"], out[n + "/T"] = E, P, np.array(c["T"])
        out[n + "/equil"] = np.array(c["equil"])
        out[n + "/params"] = np.array([c["L"], c["cutoff"], c["cage_strain"], *c["efield"], c["occupancy"]])
    np.savez_compressed(os.path.join(HERE, "ref_equilibrium.npz"), **out)


ANALYSIS_CASES = [
    dict(name="random10", X=10, Y=10, Z=10, cutoff=3, T=300),
    dict(name="spectrum", X=10, Y=12, Z=14, cutoff=3, T=150, pattern="spectrum"),
    dict(name="buckled", X=10, Y=10, Z=10, cutoff=3, T=300, pattern="buckled"),
    dict(name="slab12", X=12, Y=12, Z=1, cutoff=3, T=300),
    dict(name="mixture10", X=10, Y=10, Z=10, cutoff=3, T=250, lengths=(1.0, 0.5, 0.0), prevalence=(0.5, 0.3, 0.2)),
]


def _zero_vacancies(r):
    """Vacancies as zero vectors (the GPU build's convention) in the reference's own lattice."""
    lat = r.lattice()
    lat[lat[:, 3] == 0, :3] = 0.0
    r.set_lattice(lat)
    return lat


def _parse_rdf(path):
    rows = [l.split() for l in open(path) if l.strip() and not l.startswith("#")]
    return np.array([[float(v) for v in row] for row in rows])


def analysis(R, tmp):
    out = {}
    for c in ANALYSIS_CASES:
        r = _sim(R, c)
        if "pattern" in c:
            r.init_pattern(c["pattern"])
        n = c["name"]
        out[n + "/lattice"] = _zero_vacancies(r)
        out[n + "/shape"] = np.array([c["X"], c["Y"], c["Z"]])
        out[n + "/potential"] = r.potential_map()
        out[n + "/efield4"] = r.efield_map(4)
        out[n + "/efieldoffset2"] = r.efield_map(2, half=True)
        pol, landau = r.observables()
        out[n + "/order"] = np.array([pol, landau])
        path = os.path.join(tmp, n + "-rdf.dat")
        r.write("rdf", path)
        out[n + "/rdf"] = _parse_rdf(path)
    np.savez_compressed(os.path.join(HERE, "ref_analysis.npz"), **out)


WRITERS = ("potential_xyz", "potential_cube", "efield_xyz", "efieldoffset_xyz", "potential_pgm", "dipoles_xyz",
           "dipoles_ppm", "dipoles_svg", "rdf", "recombination")


def files(R, tmp):
    c = dict(X=10, Y=10, Z=10, cutoff=3, T=300, lengths=(1.0, 0.0), prevalence=(0.8, 0.2))
    r = _sim(R, c)
    out = {"lattice": _zero_vacancies(r), "shape": np.array([10, 10, 10]), "T": np.array(300),
           "potential": r.potential_map(), "efield4": r.efield_map(4), "efieldoffset2": r.efield_map(2, half=True)}
    for kind in WRITERS:
        path = os.path.join(tmp, "w_" + kind)
        r.write(kind, path)
        out["file/" + kind] = np.frombuffer(open(path, "rb").read(), np.uint8)
    for kind in ("dumb_terminal", "recombination"):
        path = os.path.join(tmp, "c_" + kind)
        r.capture(kind, path)
        out["stderr/" + kind] = np.frombuffer(open(path, "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_files.npz"), **out)


DRIVER_CFG = """T = 300
X = 10
Y = 12
Z = 14
InitialLattice = "spectrum"
Efield: { x = 0.0; y = 0.0; z = 0.0; }
DipoleCutOff = 3
ConstrainToX = false
K = 0.0
Dipoles = [ 1.0 ];
Prevalence = [ 1.0 ];
CageStrain = 1.0
MCMegaSteps = 0
MCEqmSteps = 0
MCMoves = 1.0
DisplayDumbTerminal = false
CalculateRecombination = false
CalculateRadialOrderParameter = true
CalculatePotential = true
CalculateEfield = true
SaveDipolesPNG = true
SaveDipolesSVG = true
SaveDipolesXYZ = true
SavePotentialCube = true
"""


def driver_files(tmp):
    """Run the stock reference binary (oracle/_ref/starrynight) in a scratch directory."""
    import subprocess
    exe = os.path.join(ROOT, "oracle", "_ref", "starrynight")
    d = os.path.join(tmp, "driver")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "starrynight.cfg"), "w") as f:
        f.write(DRIVER_CFG)
    subprocess.run([exe], cwd=d, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    out = {"cfg": np.frombuffer(DRIVER_CFG.encode(), np.uint8)}
    for name in sorted(os.listdir(d)):
        if name in ("starrynight.cfg",) or name.endswith(".log"):
            continue
        out["file/" + name] = np.frombuffer(open(os.path.join(d, name), "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_driver_files.npz"), **out)


def main():
    from oracle import oracle as O
    from oracle import ref_harness as R
    O.build(ref=True)
    if not R.available():
        raise SystemExit("the reference harness is not built (reference tree missing?)")
    import tempfile
    if "--equilibrium-only" in sys.argv:
        # optional case names after the flag: run only those again
        rest = sys.argv[sys.argv.index("--equilibrium-only") + 1:]
        equilibrium([a for a in rest if not a.startswith("-")] or None)
        return
    if "--analysis-only" not in sys.argv:
        neighbours(R)
        trajectories(R)
        site_energies(R)
    with tempfile.TemporaryDirectory() as tmp:
        analysis(R, tmp)
        files(R, tmp)
        driver_files(tmp)
    if "--analysis-only" in sys.argv:
        return
    if "--skip-equilibrium" not in sys.argv:
        equilibrium()


if __name__ == "__main__":
    main()
