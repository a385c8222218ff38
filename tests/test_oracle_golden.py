"""The CPU oracle against vectors produced by the unmodified reference
(tests/golden/, generated by make_golden.py) and against published
known-answer values.  No GPU needed."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al. SC'11)
    assert [hex(v) for v in O.philox([0, 0, 0, 0], [0, 0])] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_mt19937_known_answer():
    # first outputs of MT19937 with the default seed 5489 (Matsumoto & Nishimura)
    g = O.MTState(5489)
    assert [g.u32() for _ in range(3)] == [3499211612, 581869302, 3890346734]


def test_neighbour_tables_match_reference():
    d = np.load(os.path.join(GOLD, "ref_neighbours.npz"))
    for rc in range(1, 7):
        for tag, Z in (("3d", 8 * rc + 1), ("2d", 1)):
            dxyz, dist = O.neighbours(rc, Z)
            assert np.array_equal(dxyz, d["rc%d_%s_dxyz" % (rc, tag)])
            assert np.array_equal(dist, d["rc%d_%s_d" % (rc, tag)])


TRAJ = ["cube8", "field_K", "slab", "constrain_x", "vacancies", "mixture_rc4"]
CFG = {
    "cube8": dict(X=8, Y=8, Z=8, cutoff=3, T=300, moves=20000),
    "field_K": dict(X=6, Y=8, Z=10, cutoff=2, T=150, efield=(0.1, -0.2, 0.3), K=0.5, cage_strain=0.7, moves=20000),
    "slab": dict(X=12, Y=12, Z=1, cutoff=3, T=300, moves=20000),
    "constrain_x": dict(X=8, Y=8, Z=8, cutoff=3, T=300, constrain_to_x=True, moves=20000),
    "vacancies": dict(X=8, Y=8, Z=8, cutoff=3, T=200, lengths=(1.0, 0.0), prevalence=(0.7, 0.3), moves=20000),
    "mixture_rc4": dict(X=10, Y=10, Z=10, cutoff=4, T=250, lengths=(1.0, 0.5, 0.0), prevalence=(0.5, 0.3, 0.2),
                        efield=(0.0, 0.0, 0.2), moves=8000),
}


@pytest.mark.parametrize("name", TRAJ)
def test_random_sequential_trajectory_is_bit_exact(name):
    d = np.load(os.path.join(GOLD, "ref_trajectories.npz"))
    c = CFG[name]
    m = O.make_model(c["X"], c["Y"], c["Z"], c["cutoff"], T=c["T"], efield=c.get("efield", (0, 0, 0)),
                     K=c.get("K", 0.0), cage_strain=c.get("cage_strain", 1.0),
                     constrain_to_x=c.get("constrain_to_x", False))
    assert m.beta == float(d[name + "_beta"])
    mt = O.MTState((0xDEADBEEF + c["T"]) & 0xFFFFFFFF)
    lat = O.ref_init_random(m, mt, c.get("lengths", (1.0,)), c.get("prevalence", (1.0,)))
    assert np.array_equal(lat, d[name + "_init"])
    acc, rej = O.ref_mc_moves(m, lat, mt, c["moves"])
    assert np.array_equal(lat, d[name + "_final"])
    assert (acc, rej) == tuple(int(v) for v in d[name + "_counts"])


def test_reference_site_energy_values():
    d = np.load(os.path.join(GOLD, "ref_site_energy.npz"))
    X, Y, Z, rc, T, ex, ey, ez, K, C = d["params"]
    m = O.make_model(int(X), int(Y), int(Z), int(rc), T=int(T), efield=(ex, ey, ez), K=K, cage_strain=C)
    lat = d["lattice"]
    for (x, y, z), v, dE in zip(d["sites"], d["new"], d["dE"]):
        new4 = np.array([v[0], v[1], v[2], 0.0], np.float32)
        assert O.ref_site_energy(m, lat, int(x), int(y), int(z), new4) == dE  # bit-exact restatement
        # the FP64 restatement (oracle b) agrees to FP32 rounding of the reference's float terms
        px, py, pz, ln = O.soa(lat)
        i = (int(x) * int(Y) + int(y)) * int(Z) + int(z)
        d64 = O.delta_energy64(m, px, py, pz, ln, i, v)
        assert abs(d64 - dE) <= 1e-5 * max(1.0, abs(dE))


def test_equilibrium_fixture_is_sane():
    d = np.load(os.path.join(GOLD, "ref_equilibrium.npz"))
    for case in ("plain", "vacfield", "rc4cage"):
        E = d[case + "/E"]
        assert E.shape == (len(d[case + "/T"]), int(d["seeds"]), int(d["prod"]))
        assert np.isfinite(E).all() and np.isfinite(d[case + "/P"]).all()
        assert np.all(np.diff(E.mean(axis=(1, 2))) > 0)  # energy per site rises with temperature
