"""The energy entry point that allocates no device memory
(sn_gpu_energy_noalloc), for callers that may not call cudaMalloc -- e.g. a
plugin whose host framework owns the device memory pool.  It reads a lattice
from the caller's own device buffers and keeps all its scratch in a fixed
array inside the library.

This file is collected last on purpose: if the check fails, a run that stops
at the first failure has already run every other test.  It passes run alone
in a fresh process and after the rest of the suite."""
import ctypes

import numpy as np
import pytest

REL_TOL = 1e-9  # FP64 reduction order differs between launches: agree to 1e-9 relative


def _lattice(sn, shape, params):
    with sn.Simulation(params, [sn.Replica(*shape, T=150.0, seed=params.seed)]) as sim:
        sim.init_lattice(0)
        sim.sweep(2)
        E_ref = sim.energy(0, "fp32")
        xyz, ln = sim.download(0)
    return xyz, ln, E_ref


@pytest.mark.gpu
def test_energy_without_allocation_matches_energy(native_lib):
    import torch
    sn = native_lib
    from starrynight_gb300 import _abi
    L = _abi.lib()
    cases = [
        ((32, 32, 32), sn.ModelParams(cutoff=3, efield=(0.0, 0.0, 0.1), dipoles=(1.0, 0.0), prevalence=(0.7, 0.3),
                                      seed=5)),
        ((24, 16, 20), sn.ModelParams(cutoff=2, cage_strain=0.5, K=0.3, efield=(0.05, 0.0, 0.05), seed=6)),
    ]
    for shape, params in cases:
        xyz, ln, E_ref = _lattice(sn, shape, params)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (xyz[:, 0], xyz[:, 1], xyz[:, 2], ln)]
        torch.cuda.synchronize()
        cp = params.to_c()
        for _ in range(2):  # two calls in a row share the library's scratch array
            E = ctypes.c_double(0.0)
            st = L.sn_gpu_energy_noalloc(*[ctypes.c_void_p(t.data_ptr()) for t in dev], *shape, ctypes.byref(cp),
                                         None, ctypes.byref(E), None)
            assert st == 0, L.sn_gpu_last_error(None)
            assert abs(E.value - E_ref) <= REL_TOL * abs(E_ref), (E.value, E_ref)


@pytest.mark.gpu
def test_energy_without_allocation_rejects_oversized_lattice(native_lib):
    import torch
    sn = native_lib
    from starrynight_gb300 import _abi
    L = _abi.lib()
    buf = torch.zeros(8, device="cuda")
    cp = sn.ModelParams(cutoff=3).to_c()
    E = ctypes.c_double(0.0)
    p = ctypes.c_void_p(buf.data_ptr())
    # 1024^3 needs far more than 65536 tiles: refused before any device access
    st = L.sn_gpu_energy_noalloc(p, p, p, p, 1024, 1024, 1024, ctypes.byref(cp), None, ctypes.byref(E), None)
    assert st == 1  # SN_ERR_ARG
    assert b"at most 65536" in L.sn_gpu_last_error(None)
