"""libsn_io (include/sn_io.h): the reference's analysis file formats written
from arrays must be byte-identical to the files the reference's own writers
produce from the same lattice (tests/golden/ref_files.npz); checkpoints
round-trip and reject corrupt or mismatched files."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from starrynight_gb300 import formats as F

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_files.npz"))
LAT = GOLD["lattice"]
SHAPE = tuple(int(v) for v in GOLD["shape"])
T = int(GOLD["T"])
XYZ = np.ascontiguousarray(LAT[:, :3])


def _ref(key):
    return GOLD[key].tobytes()


def _read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("kind,writer,data", [
    ("potential_xyz", F.write_potential_xyz, "potential"),
    ("potential_cube", F.write_potential_cube, "potential"),
    ("potential_pgm", F.write_potential_pgm, "potential"),
    ("efield_xyz", F.write_field_xyz, "efield4"),
    ("efieldoffset_xyz", F.write_field_xyz, "efieldoffset2"),
])
def test_map_writers_byte_identical(tmp_path, kind, writer, data):
    p = str(tmp_path / kind)
    writer(p, SHAPE, GOLD[data])
    assert _read(p) == _ref("file/" + kind)


@pytest.mark.parametrize("kind,writer", [
    ("dipoles_xyz", F.write_dipoles_xyz),
    ("dipoles_ppm", F.write_dipoles_ppm),
    ("dipoles_svg", F.write_dipoles_svg),
])
def test_lattice_writers_byte_identical(tmp_path, kind, writer):
    p = str(tmp_path / kind)
    writer(p, SHAPE, XYZ)
    assert _read(p) == _ref("file/" + kind)


def test_maps_from_oracle_match_reference_maps():
    # the writers' inputs here are the reference's maps; the oracle (and the GPU) give the same bits
    pot = O.potential_map(LAT[:, 0], LAT[:, 1], LAT[:, 2], LAT[:, 3], SHAPE, 6)
    assert np.array_equal(pot, GOLD["potential"])


def test_rdf_file(tmp_path):
    p = str(tmp_path / "rdf.dat")
    fe, afe, cnt = O.radial_order(LAT[:, 0], LAT[:, 1], LAT[:, 2], SHAPE, 9, float_sums=True)
    F.append_rdf(p, 9, fe.astype(np.float32).astype(np.float64), afe.astype(np.float32).astype(np.float64), cnt, T)
    mine, ref = _read(p).decode().splitlines(), _ref("file/rdf").decode().splitlines()
    assert len(mine) == len(ref)
    assert mine[0] == ref[0] and mine[-1] == ref[-1] == ""
    for a, b in zip(mine[1:-1], ref[1:-1]):
        ra, rb = a.split(), b.split()
        # r^2, r, count, T exactly; the means to the float sum's last printed digit
        assert [ra[i] for i in (0, 1, 4, 5)] == [rb[i] for i in (0, 1, 4, 5)]
        assert abs(float(ra[2]) - float(rb[2])) <= 2e-6 and abs(float(ra[3]) - float(rb[3])) <= 2e-6
    # appending adds a second data set
    F.append_rdf(p, 9, fe, afe, cnt, T)
    assert len(_read(p).decode().splitlines()) == 2 * len(ref)


def test_recombination_log_and_art(tmp_path):
    p = str(tmp_path / "rec_log")
    F.recombination(p, SHAPE, GOLD["potential"], T, art=False)
    assert _read(p) == _ref("file/recombination")
    p2 = str(tmp_path / "rec_art")
    F.recombination(p2, SHAPE, GOLD["potential"], T, art=True)
    assert _read(p2) == _ref("stderr/recombination")


def test_dumb_terminal(tmp_path):
    p = str(tmp_path / "term")
    dmax = F.dumb_terminal(p, SHAPE, XYZ, LAT[:, 3], GOLD["potential"], T)
    assert _read(p) == _ref("stderr/dumb_terminal")
    z0 = GOLD["potential"].reshape(SHAPE)[:, :, 0]
    assert dmax == pytest.approx(float(np.abs(z0.astype(np.float32)).max()))


def _header():
    return dict(X=SHAPE[0], Y=SHAPE[1], Z=SHAPE[2], cutoff=3, sweeps=123456789012, seed=0xDEADBEEF + 300, T=300.0,
                efield=(0.0, 0.1, -0.2), accept=77, attempt=1000)


def test_checkpoint_round_trip(tmp_path):
    p = str(tmp_path / "ck.bin")
    F.write_checkpoint(p, _header(), XYZ, LAT[:, 3])
    h, xyz, ln = F.read_checkpoint(p)
    want = _header()
    for k, v in want.items():
        assert h[k] == (tuple(v) if k == "efield" else v), k
    assert np.array_equal(xyz, XYZ) and np.array_equal(ln, LAT[:, 3])
    h2, _, _ = F.read_checkpoint(p, shape=SHAPE)
    assert h2["sweeps"] == want["sweeps"]


def test_checkpoint_rejects_corruption_and_size(tmp_path):
    p = str(tmp_path / "ck.bin")
    F.write_checkpoint(p, _header(), XYZ, LAT[:, 3])
    with pytest.raises(ValueError, match="different lattice size"):
        F.read_checkpoint(p, shape=(SHAPE[0], SHAPE[1], SHAPE[2] + 2))
    raw = bytearray(_read(p))
    raw[200] ^= 0x01  # one bit of the lattice payload
    bad = str(tmp_path / "bad.bin")
    with open(bad, "wb") as f:
        f.write(bytes(raw))
    with pytest.raises(ValueError, match="corrupt"):
        F.read_checkpoint(bad)
    with open(bad, "wb") as f:
        f.write(b"not a checkpoint at all")
    with pytest.raises(ValueError, match="not a checkpoint"):
        F.read_checkpoint(bad)
    with open(bad, "wb") as f:
        f.write(bytes(raw[: len(raw) // 2]))  # truncated
    with pytest.raises(ValueError):
        F.read_checkpoint(bad)
