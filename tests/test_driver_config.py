"""The C host driver's configuration handling (no GPU needed): the
libconfig-subset reader with the reference's key set and lookup rules
(src/starrynight-config.c:98-182) and the argv overrides of
src/starrynight-main.c:142-151."""
import os
import subprocess

import pytest

CFG = r'''# test configuration, libconfig syntax
LOGFILE = "ignored.log";   // shadowed by the driver, as in the reference
T: 150
X = 12; Y = 10
Z = 8,
Efield:
{
  x = 0.5;   /* block comment */
  y = -0.25
  z = 1e-1
}
K: 0.75
CageStrain = 2.5
Dipoles    = [ 1.0, 0.5, 0.0 ];
Prevalence = [ 0.5, 0.25, 0.25 ];
ConstrainToX: TRUE
DipoleCutOff: 2
InitialLattice = "ferro" "_wall"   # adjacent strings concatenate
MCEqmSteps: 3
MCMegaSteps: 0x10
MCMoves: 4.0
SaveDipolesXYZ: false
'''


def run(tmp_path, text, *args):
    import starrynight_gb300 as sn
    sn.build()
    p = tmp_path / "starrynight.cfg"
    p.write_text(text)
    r = subprocess.run([sn.driver_path(), "--print-config", *args], cwd=tmp_path, capture_output=True, text=True)
    vals = {}
    for line in r.stdout.splitlines():
        k, _, v = line.partition(" ")
        vals[k] = v
    return r, vals


def test_reads_reference_keys(tmp_path):
    r, v = run(tmp_path, CFG)
    assert r.returncode == 0, r.stderr
    assert v["T"] == "150" and (v["X"], v["Y"], v["Z"]) == ("12", "10", "8")
    assert v["Efield"] == "0.5 -0.25 0.1"
    assert v["K"] == "0.75" and v["CageStrain"] == "2.5" and v["DipoleCutOff"] == "2"
    assert v["Dipoles"] == "1 0.5 0" and v["Prevalence"] == "0.5 0.25 0.25"
    assert v["ConstrainToX"] == "1" and v["InitialLattice"] == "ferro_wall"
    assert (v["MCEqmSteps"], v["MCMegaSteps"], v["MCMoves"]) == ("3", "16", "4")
    assert v["Seed"] == str((0xDEADBEEF + 150) & 0xFFFFFFFF)  # src/starrynight-main.c:172


def test_argv_overrides_temperature_and_cage_strain(tmp_path):
    r, v = run(tmp_path, CFG, "400", "0.5")
    assert v["T"] == "400" and v["CageStrain"] == "0.5"
    assert v["Seed"] == str((0xDEADBEEF + 400) & 0xFFFFFFFF)


def test_lookups_are_type_strict_like_libconfig(tmp_path):
    # an int where the reference looks up a float is not read (no autoconvert)
    r, v = run(tmp_path, "CageStrain = 3\nK = 2\nT = 300.0\n")
    assert v["CageStrain"] == "1" and v["K"] == "1"  # reference defaults
    assert v["T"] == "300"


def test_autotune_key(tmp_path):
    r, v = run(tmp_path, "AutoTune = 4\n")
    assert r.returncode == 0 and v["AutoTune"] == "4"
    r, v = run(tmp_path, "X = 8\n")
    assert v["AutoTune"] == "0"


def test_single_species_spelling(tmp_path):
    r, v = run(tmp_path, "Dipole = 1.5\nDipoleFraction = 0.7\nSeed = 99\n")
    assert v["Dipoles"] == "1.5 0" and v["Prevalence"] == "0.7 0.3" and v["Seed"] == "99"


@pytest.mark.parametrize("bad,line", [("T = \n", 2), ("X = 3\nY = [1, \"a\"]\n", 2), ("Efield: { x = 1.0 \n", 2),
                                      ("X = 1\nX = 2\n", 2), ("/* open comment\n", 1)])
def test_syntax_errors_report_a_line(tmp_path, bad, line):
    r, v = run(tmp_path, bad)
    assert r.returncode != 0
    assert ":%d - " % line in r.stderr or ":%d" % line in r.stderr, r.stderr


def test_missing_file_is_an_error(tmp_path):
    import starrynight_gb300 as sn
    sn.build()
    r = subprocess.run([sn.driver_path(), "--print-config"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "I/O" in r.stderr
