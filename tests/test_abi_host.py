"""The C-ABI library loads on a machine without a GPU, exports every entry
point declared in include/sn_gpu.h, and its host-only planner produces
conflict-free schedules.  No compute call is made here."""
import ctypes

import pytest

import starrynight_gb300 as sn
from starrynight_gb300 import _abi


def test_library_exports_every_declared_symbol(native_lib):
    L = ctypes.CDLL(sn.lib_path())
    names = _abi.exported_names()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(native_lib):
    L = _abi.lib()
    assert L.sn_gpu_status_string(0) == b"ok"
    assert b"schedule" in L.sn_gpu_status_string(3)


def test_neighbour_counts_match_gen_neighbour(native_lib):
    from oracle import oracle as O
    for rc in range(1, 7):
        for Z in (1, 40):
            assert sn.neighbour_count(rc, Z) == len(O.neighbours(rc, Z)[0])


CONFIGS = [(32, 32, 32, 3), (256, 256, 256, 3), (48, 48, 48, 3), (64, 64, 64, 3), (96, 96, 96, 3),
           (128, 128, 128, 3), (128, 128, 128, 4), (96, 96, 96, 5), (2048, 2048, 1, 5), (20, 20, 28, 3)]


@pytest.mark.parametrize("X,Y,Z,rc", CONFIGS)
def test_planner_fits_shared_memory(native_lib, X, Y, Z, rc):
    s = sn.plan_schedule(X, Y, Z, rc)
    assert s["smem_bytes"] <= 227 * 1024
    assert s["bx"] * s["nbx"] == X and s["by"] * s["nby"] == Y and s["bz"] * s["nbz"] == Z
    assert min(s["bx"], s["by"]) >= rc and (Z == 1 or s["bz"] >= rc)


@pytest.mark.parametrize("X,Y,Z,rc", [(8, 8, 8, 3), (6, 6, 6, 3), (12, 12, 12, 3), (32, 32, 32, 3), (24, 24, 1, 3),
                                      (16, 16, 16, 4), (20, 20, 20, 5), (48, 36, 1, 5), (8, 12, 16, 2), (20, 20, 28, 3)])
def test_schedule_colours_never_interact(native_lib, X, Y, Z, rc):
    s = sn.plan_schedule(X, Y, Z, rc)
    assert sn.check_schedule(X, Y, Z, rc, s)


def test_check_schedule_rejects_interacting_colours(native_lib):
    s = sn.plan_schedule(16, 16, 16, 3)
    bad = dict(s, s=2)  # site-colour stride smaller than cutoff + 1
    assert not sn.check_schedule(16, 16, 16, 3, bad)
    s = sn.plan_schedule(12, 12, 12, 3)  # blocks of 6: the site colouring alone is not periodic
    assert s["bx"] % s["s"] != 0 and sn.check_schedule(12, 12, 12, 3, s)
    bad = dict(s, mx=1, my=1, mz=1)  # every block updated at once
    assert not sn.check_schedule(12, 12, 12, 3, bad)


@pytest.mark.parametrize("shape,rc", [((25, 25, 25), 3), ((30, 30, 2), 3), ((8, 8, 8), 7)])
def test_planner_reports_unschedulable_lattices(native_lib, shape, rc):
    with pytest.raises(sn.SnError) as e:
        sn.plan_schedule(*shape, rc)
    assert e.value.name in ("SN_ERR_SCHEDULE", "SN_ERR_UNSUPPORTED")
