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
