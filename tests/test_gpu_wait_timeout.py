"""The dataflow sweep's bounded waits, made to run out on purpose.

A block of the persistent sweep waits for its earlier-coloured neighbours'
done flags; every such wait gives up after a poll limit and records an error
that the host turns into SN_ERR_TIMEOUT.  The reference has no waits (it
exit()s on its own errors, src/starrynight-config.c:113-121); the status code
is this library's contract.  Here a test hook points one block's dependency
at a flag that no block ever publishes, with a short limit: the sweep must
return SN_ERR_TIMEOUT, nothing may hang or fault, and after the hook is
removed and the lattice uploaded again the handle must sweep exactly like a
fresh one."""
import time

import numpy as np
import pytest

SN_ERR_TIMEOUT = 6


@pytest.mark.gpu
def test_stalled_block_reports_timeout_and_handle_recovers(native_lib):
    sn = native_lib
    from starrynight_gb300._abi import SnError
    params = sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), seed=31)
    rep = sn.Replica(32, 32, 32, T=300.0, seed=31)
    # the undisturbed run: 1 sweep, then 3 more
    with sn.Simulation(params, [rep]) as ref:
        ref.init_lattice(0)
        ref.sweep(1)
        ref.sweep(3)
        want, _ = ref.download(0)
    with sn.Simulation(params, [rep]) as sim:
        sim.init_lattice(0)
        sim.sweep(1)
        xyz1, ln1 = sim.download(0)
        sim.set_wait_limit(2000)
        sim.test_stall_block(0)
        t0 = time.perf_counter()
        with pytest.raises(SnError) as ei:
            sim.sweep(2)
        assert ei.value.status == SN_ERR_TIMEOUT, str(ei.value)
        assert time.perf_counter() - t0 < 30.0  # the waits gave up; nothing spun for long
        # the error was reported once and cleared: the handle is usable again
        sim.test_stall_block(-1)
        sim.set_wait_limit(1 << 22)
        sim.upload(0, xyz1, ln1)
        sim.set_sweep_count(1)
        acc, rej = sim.sweep(3, counts=True)
        assert acc + rej == 3 * 32 ** 3
        got, _ = sim.download(0)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_wait_limit_and_stall_hook_reject_bad_arguments(native_lib):
    sn = native_lib
    from starrynight_gb300._abi import SnError
    with sn.Simulation(sn.ModelParams(cutoff=2, seed=3), [sn.Replica(16, 16, 16, T=300.0)]) as sim:
        with pytest.raises(SnError):
            sim.set_wait_limit(0)
        with pytest.raises(SnError):
            sim.test_stall_block(1 << 20)
        sim.init_lattice(0)
        sim.sweep(2)  # untouched by the refused calls
