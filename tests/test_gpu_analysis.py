"""GPU analysis stencils (sn_gpu_potential, sn_gpu_efield, sn_gpu_radial_order,
sn_gpu_order_parameters) against the reference's own maps
(tests/golden/ref_analysis.npz) and the oracle: the potential and E-field maps
bit for bit, the FP64 correlation sums to 1e-12, and checkpoint/resume giving
the run that never stopped."""
import os

import numpy as np
import pytest

import starrynight_gb300 as sn
from oracle import oracle as O
from starrynight_gb300 import formats as F

pytestmark = pytest.mark.gpu

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_analysis.npz"))
CASES = sorted({k.split("/")[0] for k in GOLD.files})


def _sim_for(name):
    lat = GOLD[name + "/lattice"]
    shape = tuple(int(v) for v in GOLD[name + "/shape"])
    lens = tuple(sorted({float(v) for v in lat[:, 3]}, reverse=True))
    params = sn.ModelParams(cutoff=3, dipoles=lens, prevalence=tuple(1.0 / len(lens) for _ in lens), seed=3)
    sim = sn.Simulation(params, [sn.Replica(*shape, T=300.0, seed=3)])
    sim.upload(0, lat[:, :3], lat[:, 3])
    return sim, lat, shape


@pytest.mark.parametrize("name", CASES)
def test_maps_bitwise_vs_reference(name):
    sim, lat, shape = _sim_for(name)
    with sim:
        assert np.array_equal(sim.potential(0, 6), GOLD[name + "/potential"])
        assert np.array_equal(sim.efield(0, 4), GOLD[name + "/efield4"])
        assert np.array_equal(sim.efield(0, 2, half_offset=True), GOLD[name + "/efieldoffset2"])


@pytest.mark.parametrize("name", CASES)
def test_radial_and_order_vs_oracle(name):
    sim, lat, shape = _sim_for(name)
    with sim:
        fe, afe, cnt = sim.radial_order(0, 9)
        pol, landau, s3 = sim.order_parameters(0)
    ofe, oafe, ocnt = O.radial_order(lat[:, 0], lat[:, 1], lat[:, 2], shape, 9)
    assert np.array_equal(cnt, ocnt)
    # the same float terms summed in FP64 in another order: allow 1e-10 of the bins'
    # magnitude bound count * max|p|^2 (terms are at most 4 |p_i||p_j| for AFE)
    pmax2 = float(np.max(np.sum(lat[:, :3].astype(np.float64) ** 2, axis=1)))
    bound = 1e-10 * np.maximum(cnt, 1) * 4.0 * max(pmax2, 1.0)
    err_fe, err_afe = np.abs(fe - ofe), np.abs(afe - oafe)
    assert np.all(err_fe <= bound), (err_fe.max(), int(np.argmax(err_fe / bound)), bound.min())
    assert np.all(err_afe <= bound), (err_afe.max(), int(np.argmax(err_afe / bound)), bound.min())
    opol, olandau, os3 = O.order_params(lat[:, 0], lat[:, 1], lat[:, 2])
    n = lat.shape[0]
    assert np.all(np.abs(s3 - os3) <= 1e-12 * n), (s3, os3)
    assert pol == pytest.approx(opol, abs=1e-12)
    assert landau == pytest.approx(olandau, rel=1e-10, abs=1e-9)
    # the reference's polarisation() is the same double sum of x components
    assert pol == pytest.approx(float(GOLD[name + "/order"][0]), abs=1e-12)


def test_maps_after_sweeps_match_oracle_at_64cubed():
    """A lattice the sweep produced (vacancies, mixed lengths), at a size that exercises many blocks."""
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.5, 0.0), prevalence=(0.5, 0.3, 0.2),
                            seed=11)
    with sn.Simulation(params, [sn.Replica(64, 48, 32, T=200.0, seed=11)]) as sim:
        sim.init_lattice(0)
        sim.sweep(5)
        xyz, ln = sim.download(0)
        pot = sim.potential(0, 6)
        ef = sim.efield(0, 4)
        efo = sim.efield(0, 2, half_offset=True)
    shape = (64, 48, 32)
    assert np.array_equal(pot, O.potential_map(xyz[:, 0], xyz[:, 1], xyz[:, 2], ln, shape, 6))
    assert np.array_equal(ef, O.efield_map(xyz[:, 0], xyz[:, 1], xyz[:, 2], shape, 4, False))
    assert np.array_equal(efo, O.efield_map(xyz[:, 0], xyz[:, 1], xyz[:, 2], shape, 2, True))


def test_other_cutoffs_and_errors():
    sim, lat, shape = _sim_for("random10")
    with sim:
        for c in (1, 3, 5):
            assert np.array_equal(sim.potential(0, c), O.potential_map(lat[:, 0], lat[:, 1], lat[:, 2], lat[:, 3],
                                                                        shape, c))
        with pytest.raises(sn.SnError):
            sim.potential(0, 0)
        with pytest.raises(sn.SnError):
            sim.efield(0, 33)
        with pytest.raises(sn.SnError):
            sim.radial_order(1, 9)


def test_checkpoint_resume_is_the_uninterrupted_run(tmp_path):
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.05), dipoles=(1.0, 0.0), prevalence=(0.8, 0.2), seed=21)
    rep = sn.Replica(32, 32, 32, T=150.0, seed=21)
    path = str(tmp_path / "ck.bin")
    with sn.Simulation(params, [rep]) as a:
        a.init_lattice(0)
        a.sweep(7)
        xyz, ln = a.download(0)
        F.write_checkpoint(path, dict(X=32, Y=32, Z=32, cutoff=3, sweeps=a.sweep_count(), seed=21, T=150.0,
                                      efield=(0.0, 0.0, 0.05), accept=0, attempt=0), xyz, ln)
        acc_a, rej_a = a.sweep(6, counts=True)
        end_a = a.download(0)[0]
    h, xyz2, ln2 = F.read_checkpoint(path, shape=(32, 32, 32))
    assert h["sweeps"] == 7
    with sn.Simulation(params, [rep]) as b:
        b.upload(0, xyz2, ln2)
        b.set_sweep_count(h["sweeps"])
        acc_b, rej_b = b.sweep(6, counts=True)
        end_b = b.download(0)[0]
        assert b.sweep_count() == 13
    assert (acc_a, rej_a) == (acc_b, rej_b)
    assert np.array_equal(end_a, end_b)
