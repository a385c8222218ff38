"""sn_gpu_sweep_download: the last sweep writes each block's final sites
straight into a pinned host buffer; the lattice it leaves there is the one
sn_gpu_sweep + sn_gpu_download_lattice give, bit for bit, for pinned buffers,
pageable buffers (staged download) and skipped replicas, under both sweep
schedules; no later sweep writes into the buffer again."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _table(sn):
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.5, 0.0), prevalence=(0.6, 0.2, 0.2), seed=21)
    reps = [sn.Replica(48, 32, 64, T=150.0, seed=21), sn.Replica(32, 32, 32, T=300.0, seed=22),
            sn.Replica(96, 64, 1, T=250.0, seed=23)]
    return params, reps


@pytest.mark.parametrize("schedule", ["flow", "phases"])
def test_sweep_download_equals_sweep_then_download(native_lib, monkeypatch, schedule):
    import torch
    sn = native_lib
    monkeypatch.delenv("SN_SCHEDULE", raising=False)
    if schedule == "phases":
        monkeypatch.setenv("SN_SCHEDULE", "phases")
    params, reps = _table(sn)
    with sn.Simulation(params, reps) as sim:
        for r in range(3):
            sim.init_lattice(r)
        ref_counts = sim.sweep(3, counts=True)
        ref = [sim.download(r)[0] for r in range(3)]
    with sn.Simulation(params, reps) as sim:
        for r in range(3):
            sim.init_lattice(r)
        pinned = torch.full((3 * reps[0].n_sites,), np.nan, dtype=torch.float32, pin_memory=True)
        pageable = np.full((reps[1].n_sites, 3), np.nan, np.float32)
        counts = sim.sweep_download(3, [pinned.data_ptr(), pageable, None], counts=True)
        assert counts == ref_counts
        got0 = pinned.numpy().reshape(-1, 3).copy()
        assert np.array_equal(got0, ref[0])
        assert np.array_equal(pageable, ref[1])
        # the device lattices are the same ones
        assert all(np.array_equal(sim.download(r)[0], ref[r]) for r in range(3))
        # later sweeps leave the buffer alone
        sim.sweep(2)
        assert np.array_equal(pinned.numpy().reshape(-1, 3), got0)
        assert not np.array_equal(sim.download(0)[0], got0)
        # zero sweeps: a plain download into the buffer
        zero = torch.zeros(3 * reps[2].n_sites, dtype=torch.float32, pin_memory=True)
        sim.sweep_download(0, [None, None, zero.data_ptr()])
        assert np.array_equal(zero.numpy().reshape(-1, 3), sim.download(2)[0])


def test_sweep_download_headline_lattice(native_lib):
    """256^3, p = 0.7: the pinned-buffer result equals the device lattice."""
    import torch
    sn = native_lib
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3), seed=5)
    with sn.Simulation(params, [sn.Replica(256, 256, 256, T=150.0, seed=5)]) as sim:
        sim.init_lattice(0)
        buf = torch.empty(3 * 256 ** 3, dtype=torch.float32, pin_memory=True)
        acc, rej = sim.sweep_download(2, [buf.data_ptr()], counts=True)
        assert 0 < acc < acc + rej
        assert np.array_equal(buf.numpy().reshape(-1, 3), sim.download(0)[0])


def test_abi_pinned_buffer(native_lib):
    """A buffer from sn_gpu_host_alloc (page-locked, for C hosts without CUDA
    headers) takes the in-sweep write-out."""
    import ctypes
    from starrynight_gb300._abi import lib
    sn = native_lib
    params = sn.ModelParams(cutoff=2, efield=(0.05, 0.0, 0.0), seed=9)
    rep = sn.Replica(24, 24, 24, T=200.0, seed=9)
    n = 3 * rep.n_sites
    p = lib().sn_gpu_host_alloc(4 * n)
    assert p
    try:
        with sn.Simulation(params, [rep]) as sim:
            sim.init_lattice(0)
            sim.sweep_download(2, [p])
            got = np.ctypeslib.as_array((ctypes.c_float * n).from_address(p)).reshape(-1, 3).copy()
            assert np.array_equal(got, sim.download(0)[0])
    finally:
        lib().sn_gpu_host_free(p)
