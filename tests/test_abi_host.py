"""The C-ABI library loads on a machine without a GPU, exports every entry
point declared in include/sn_gpu.h, and its host-only planner produces
conflict-free schedules.  No compute call is made here."""
import ctypes

import numpy as np
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


def test_headline_plan_keeps_two_ctas_per_sm(native_lib):
    """The 256^3 cutoff-3 lattice gets the cached-field sweep on 8x8x32 blocks
    with at most half of the SM's 228 KB of shared memory (less 1 KB reserved
    per CTA and the kernel's static slots) per CTA: two CTAs per SM, the
    occupancy the kernel is tuned for."""
    s = sn.plan_schedule(256, 256, 256, 3)
    assert s["field_cache"] == 1
    assert (s["bx"], s["by"], s["bz"]) == (8, 8, 32)
    assert s["smem_bytes"] <= (228 * 1024 - 2 * 1024) // 2 - 128


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


def _flow_tables(sn):
    rng = np.random.default_rng(777)
    sizes = rng.choice([32, 48, 64, 96, 128], size=64)
    uneven = [sn.Replica(int(L), int(L), int(L), T=100.0 + i, seed=i) for i, L in enumerate(sizes)]
    mixed_2d = [sn.Replica(96, 96, 96, T=300.0)] * 3 + [sn.Replica(2048, 2048, 1, T=300.0),
                                                         sn.Replica(40, 64, 1, T=200.0)]
    odd = [sn.Replica(10, 12, 14), sn.Replica(12, 12, 1), sn.Replica(24, 16, 20), sn.Replica(256, 256, 256)]
    return [("uneven64_rc3", sn.ModelParams(cutoff=3), uneven), ("cubes_and_slabs_rc5", sn.ModelParams(cutoff=5),
                                                                   mixed_2d),
            ("small_rc3_mixed", sn.ModelParams(cutoff=3, dipoles=(1.0, 0.5, 0.0), prevalence=(0.5, 0.3, 0.2)), odd),
            ("rc1", sn.ModelParams(cutoff=1), odd)]


def test_dataflow_schedule_is_complete_and_acyclic(native_lib):
    """Every block of every replica once; each waits exactly on its adjacent blocks of
    earlier colour, all earlier in the queue -- including tables of replicas of
    different shapes, whose block indices must not alias."""
    sn = native_lib
    for name, params, reps in _flow_tables(sn):
        st = sn.check_flow(params, reps)
        assert st["blocks"] == sum(int(np.prod([r.X, r.Y, r.Z])) // int(np.prod(
            [sn.plan_schedule(r.X, r.Y, r.Z, params.cutoff, mixed=len({d for d in params.dipoles if d > 0}) > 1)[k]
             for k in ("bx", "by", "bz")])) for r in reps), name
        assert 0 < st["max_dependencies"] <= 26, name  # the 26 neighbours of a last-colour block


def test_plan_candidates_and_forced_shapes(native_lib):
    """The candidate list starts with the planner's choice, every candidate is a
    conflict-free schedule, and a replica can be given any of them -- but not a shape
    that does not tile its lattice."""
    sn = native_lib
    for (X, Y, Z), rc, mixed in (((256, 256, 256), 3, False), ((96, 96, 96), 5, False), ((64, 48, 32), 3, True),
                                 ((2048, 2048, 1), 5, False)):
        cands = sn.plan_candidates(X, Y, Z, rc, mixed, max_out=6)
        assert 1 <= len(cands) <= 6
        assert cands[0] == sn.plan_schedule(X, Y, Z, rc, mixed)
        shapes = [(c["bx"], c["by"], c["bz"]) for c in cands]
        assert len(set(shapes)) == len(shapes)
        params = sn.ModelParams(cutoff=rc, dipoles=(1.0, 0.5) if mixed else (1.0,),
                                prevalence=(0.5, 0.5) if mixed else (1.0,))
        for c, shape in zip(cands, shapes):
            if X * Y * Z <= 100_000:  # brute-force check, small lattices only
                assert sn.check_schedule(X, Y, Z, rc, c)
            st = sn.check_flow(params, [sn.Replica(X, Y, Z, block=shape)])
            assert st["blocks"] == (X // shape[0]) * (Y // shape[1]) * (Z // shape[2])
    with pytest.raises(sn.SnError, match="does not tile"):
        sn.check_flow(sn.ModelParams(cutoff=3), [sn.Replica(64, 64, 64, block=(5, 8, 8))])


def test_host_alloc_without_a_device_is_null_not_a_crash(native_lib):
    L = _abi.lib()
    assert not L.sn_gpu_host_alloc(0)
    p = L.sn_gpu_host_alloc(64)  # NULL here (no GPU); a pointer where one exists
    L.sn_gpu_host_free(p)
    L.sn_gpu_host_free(None)
