"""The C host driver end to end on the GPU: the reference's megastep loop
with its progress lines and one line of observables per megastep."""
import subprocess

import numpy as np
import pytest

CFG = """T: %d
X = 16
Y = 16
Z = 16
Efield: { x = 0.0; y = 0.0; z = 0.1; }
K: 0.0
CageStrain = 1.0
Dipoles = [1.0, 0.0]
Prevalence = [0.8, 0.2]
ConstrainToX: false
DipoleCutOff: 3
InitialLattice = "%s"
MCEqmSteps: 2
MCMegaSteps: 4
MCMoves: 3.0
SaveDipolesXYZ: %s
"""


@pytest.mark.gpu
@pytest.mark.parametrize("pattern", ["random", "ferroelectric", "buckled", "antiferro_wall", "ferro_wall",
                                     "antiferro_slip", "spectrum", "slab_delete"])
def test_driver_runs_megasteps(native_lib, tmp_path, pattern):
    xyz = "true" if pattern == "random" else "false"
    (tmp_path / "starrynight.cfg").write_text(CFG % (300, pattern, xyz))
    r = subprocess.run([native_lib.driver_path()], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [l.split() for l in r.stdout.splitlines() if not l.startswith("#")]
    assert len(rows) == 4
    data = np.array(rows, float)
    assert np.array_equal(data[:, 1], [9, 12, 15, 18])  # (eqm + i + 1) * 3 sweeps
    assert np.all(np.isfinite(data[:, 2])) and np.all(data[:, 3] >= 0)
    assert r.stderr.count("MC Moves (per second):") == 4
    tail = [l for l in r.stderr.splitlines() if l.startswith("Monte Carlo moves - ACCEPT:")][0]
    acc, rej = int(tail.split()[5]), int(tail.split()[7])
    assert 0 < acc < acc + rej
    if xyz == "true":
        lines = (tmp_path / "initial_dipoles.xyz").read_text().splitlines()
        assert lines[0] == str(2 * 16 ** 3) and len(lines) == 2 + 2 * 16 ** 3
        assert lines[2].startswith("C ") and lines[3].startswith("N ")


REF_FILES = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                               "ref_driver_files.npz"))


@pytest.mark.gpu
def test_driver_analysis_files_match_reference_binary(native_lib, tmp_path):
    """The stock reference binary and this driver on the same starrynight.cfg (a deterministic
    "spectrum" lattice, every analysis flag on, no moves) write the same files."""
    (tmp_path / "starrynight.cfg").write_bytes(REF_FILES["cfg"].tobytes())
    r = subprocess.run([native_lib.driver_path()], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    names = sorted(k[5:] for k in REF_FILES.files if k.startswith("file/"))
    assert "initial_lattice_potential.cube" in names and "rdf.dat" in names
    for name in names:
        mine = (tmp_path / name).read_bytes()
        ref = REF_FILES["file/" + name].tobytes()
        if name == "rdf.dat":  # the reference's histogram sums are float, these FP64
            a, b = mine.decode().splitlines(), ref.decode().splitlines()
            assert len(a) == len(b) and a[0] == b[0]
            for la, lb in zip(a[1:], b[1:]):
                if not lb:
                    assert not la
                    continue
                fa, fb = la.split(), lb.split()
                assert [fa[i] for i in (0, 1, 4, 5)] == [fb[i] for i in (0, 1, 4, 5)]
                assert abs(float(fa[2]) - float(fb[2])) < 2e-4 and abs(float(fa[3]) - float(fb[3])) < 2e-4
        else:
            assert mine == ref, name


@pytest.mark.gpu
def test_driver_checkpoint_resume(native_lib, tmp_path):
    """MCMegaSteps 4 in one run equals 2 + a resumed 2 (CheckpointFile / ResumeFrom)."""
    base = CFG % (300, "random", "false") + "DisplayDumbTerminal: false\nCalculateRecombination: false\n"
    one = tmp_path / "one"
    one.mkdir()
    (one / "starrynight.cfg").write_text(base.replace("MCMegaSteps: 4", "MCMegaSteps: 4") +
                                         'CheckpointFile = "end.ck"\n')
    two = tmp_path / "two"
    two.mkdir()
    (two / "starrynight.cfg").write_text(base.replace("MCMegaSteps: 4", "MCMegaSteps: 2") +
                                         'CheckpointFile = "half.ck"\n')
    three = tmp_path / "three"
    three.mkdir()
    (three / "starrynight.cfg").write_text(base.replace("MCMegaSteps: 4", "MCMegaSteps: 2")
                                           .replace("MCEqmSteps: 2", "MCEqmSteps: 0") +
                                           'ResumeFrom = "../two/half.ck"\nCheckpointFile = "end.ck"\n')
    for d in (one, two, three):
        r = subprocess.run([native_lib.driver_path()], cwd=d, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
    from starrynight_gb300 import formats as F
    h1, x1, l1 = F.read_checkpoint(str(one / "end.ck"))
    h3, x3, l3 = F.read_checkpoint(str(three / "end.ck"))
    assert h1["sweeps"] == h3["sweeps"] == (2 + 4) * 3
    assert np.array_equal(x1, x3) and np.array_equal(l1, l3)
