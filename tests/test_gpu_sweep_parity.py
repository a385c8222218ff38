"""Oracle (a): the CUDA colour sweep against the CPU mirror of the same
schedule, driven by the same Philox stream.

The proposals are bit-identical (only correctly rounded + - * / sqrt are used
on both sides), so every accepted move writes the same bits.  The accept
decisions must agree at every site except where the FP64 energy change lies
within TOL of the threshold -kT ln u (FP32 local-field rounding, or the
field cache's fixed-point grid, decides those).  After each sweep the oracle
adopts the GPU's decision at such borderline sites and the lattices must then
be bit-identical.

Both sweep methods are checked: CASES force the stencil sweep, CACHED_CASES
the cached-field sweep, which must also keep its field cache equal to a
fresh field pass after every sweep.
"""
import numpy as np
import pytest

TOL = 1e-4  # |dE_64 - (-kT ln u)| band, energy units of k_B*300K

CASES = [
    # name, (X,Y,Z), cutoff, T, efield, K, cage, dipoles, prevalence, constrain, dim, sweeps
    ("cube8_rc3", (8, 8, 8), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 3, 4),
    ("cube12_field", (12, 12, 12), 3, 150.0, (0.0, 0.0, 0.1), 0.0, 1.0, (1.0,), (1.0,), False, 3, 3),
    ("vacancy16", (16, 16, 16), 3, 150.0, (0.0, 0.0, 0.1), 0.0, 1.0, (1.0, 0.0), (0.7, 0.3), False, 3, 3),
    ("config1_32", (32, 32, 32), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 3, 10),
    ("rc2_K_aniso", (8, 12, 16), 2, 200.0, (0.1, -0.2, 0.3), 0.5, 0.7, (1.0,), (1.0,), False, 3, 3),
    ("rc4", (16, 16, 16), 4, 300.0, (0.05, 0.0, 0.05), 0.0, 0.5, (1.0, 0.0), (0.9, 0.1), False, 3, 2),
    ("rc5", (20, 20, 20), 5, 300.0, (0.0, 0.0, 0.3), 0.0, 1.0, (1.0,), (1.0,), False, 3, 2),
    ("slab2d", (24, 24, 1), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 3, 4),
    ("slab2d_rc5", (48, 36, 1), 5, 300.0, (0.0, 0.0, 0.1), 0.0, 1.0, (1.0,), (1.0,), False, 3, 3),
    ("constrain_x", (8, 8, 8), 3, 300.0, (0.2, 0, 0), 0.0, 1.0, (1.0,), (1.0,), True, 3, 3),
    ("circle_dim2", (8, 8, 8), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 2, 3),
    ("mixture", (12, 12, 12), 3, 300.0, (0, 0, 0.1), 0.0, 1.0, (1.0, 0.5, 0.0), (0.5, 0.3, 0.2), False, 3, 3),
    ("length2", (8, 8, 8), 3, 300.0, (0, 0, 0), 0.0, 1.0, (2.0,), (1.0,), False, 3, 3),
    ("rc1", (8, 12, 8), 1, 300.0, (0.0, 0.1, 0.0), 0.0, 1.0, (1.0, 0.0), (0.8, 0.2), False, 3, 3),
    ("rc6", (24, 24, 24), 6, 300.0, (0.0, 0.0, 0.1), 0.0, 1.0, (1.0,), (1.0,), False, 3, 2),
]


CACHED_CASES = [
    ("c_vacancy16", (16, 16, 16), 3, 150.0, (0.0, 0.0, 0.1), 0.0, 1.0, (1.0, 0.0), (0.7, 0.3), False, 3, 3),
    ("c_config1_32", (32, 32, 32), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 3, 10),
    ("c_rc2_K_aniso", (8, 16, 16), 2, 200.0, (0.1, -0.2, 0.3), 0.5, 0.7, (1.0,), (1.0,), False, 3, 3),
    ("c_rc4", (16, 16, 16), 4, 300.0, (0.05, 0.0, 0.05), 0.0, 0.5, (1.0, 0.0), (0.9, 0.1), False, 3, 2),
    ("c_rc5", (24, 24, 24), 5, 300.0, (0.0, 0.0, 0.3), 0.0, 1.0, (1.0,), (1.0,), False, 3, 2),
    ("c_constrain_x", (16, 16, 16), 3, 300.0, (0.2, 0, 0), 0.0, 1.0, (1.0,), (1.0,), True, 3, 3),
    ("c_circle_dim2", (16, 16, 16), 3, 300.0, (0, 0, 0), 0.0, 1.0, (1.0,), (1.0,), False, 2, 3),
    ("c_mixture", (16, 16, 16), 3, 300.0, (0, 0, 0.1), 0.0, 1.0, (1.0, 0.5, 0.0), (0.5, 0.3, 0.2), False, 3, 3),
    ("c_rc4_mixture", (16, 16, 16), 4, 300.0, (0.05, 0.0, 0.05), 0.0, 0.5, (1.0, 0.5, 0.0), (0.5, 0.3, 0.2), False, 3,
     2),
    ("c_length2", (16, 16, 16), 3, 300.0, (0, 0, 0), 0.0, 1.0, (2.0,), (1.0,), False, 3, 3),
    ("c_rc1", (8, 12, 8), 1, 300.0, (0.0, 0.1, 0.0), 0.0, 1.0, (1.0, 0.0), (0.8, 0.2), False, 3, 3),
]


def run_case(sn, O, case, seed=12345, method="stencil"):
    name, (X, Y, Z), rc, T, E, K, C, dip, prev, cx, dim, n_sweeps = case
    params = sn.ModelParams(cutoff=rc, cage_strain=C, K=K, efield=E, dipoles=dip, prevalence=prev,
                            constrain_to_x=cx, dim=dim, seed=seed, sweep_method=method)
    with sn.Simulation(params, [sn.Replica(X, Y, Z, T=T, seed=seed)]) as sim:
        cached = sim.schedule(0)["field_cache"] == 1
        assert cached == (method == "cached" and Z > 1), (name, method)
        sim.init_lattice(0)
        xyz, ln = sim.download(0)
        px, py, pz = (np.ascontiguousarray(xyz[:, k]) for k in range(3))
        sched = O.make_schedule(sim.schedule(0))
        m = O.make_model(X, Y, Z, rc, T=T, efield=E, K=K, cage_strain=C, constrain_to_x=cx, dim=dim)
        beta32 = np.float32(300.0 / T)
        nz = sorted(set(float(d) for d in dip if d > 0))
        st = O.make_stream(seed, float(beta32), nz[0] if len(nz) == 1 else 0.0)
        tot_border = tot_moves = 0
        for s in range(n_sweeps):
            acc, rej = sim.sweep(1, counts=True)
            g, _ = sim.download(0)
            res = O.colour_sweep(m, sched, st, s, px, py, pz, ln,
                                 gpu_after=(g[:, 0], g[:, 1], g[:, 2]), tol=TOL)
            assert res.hard == 0, "%s sweep %d: %d decisions outside the FP32 band" % (name, s, res.hard)
            assert np.array_equal(px, g[:, 0]) and np.array_equal(py, g[:, 1]) and np.array_equal(pz, g[:, 2])
            assert res.accepted == acc, (res.accepted, acc)
            assert acc + rej == int((ln > 0).sum())
            if cached:
                assert sim.field_cache_check(0) == 0, "%s sweep %d: field cache differs from a fresh pass" % (name, s)
            tot_border += res.borderline
            tot_moves += acc + rej
        assert tot_border <= max(2, tot_moves // 1000)
        return tot_moves, tot_border


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_sweep_accept_for_accept(native_lib, oracle_mod, case):
    run_case(native_lib, oracle_mod, case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CACHED_CASES, ids=[c[0] for c in CACHED_CASES])
def test_cached_sweep_accept_for_accept(native_lib, oracle_mod, case):
    run_case(native_lib, oracle_mod, case, method="cached")
