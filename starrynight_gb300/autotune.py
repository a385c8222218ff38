"""Empirical tile/colour-schedule autotuner.

The planner (``plan_candidates``) ranks the feasible block shapes of a
lattice by a model -- largest blocks that fit two CTAs per SM, least halo,
conflict-free shared-memory strides.  ``tune`` times the top candidates on
the GPU (CUDA events around whole sweeps, after warm-up) and returns the
fastest shape; ``tune_table`` does so once per distinct lattice size of a
replica table (optionally remembering choices in a JSON cache file) and
returns the table with every replica's ``block`` set.  ``tune_native`` makes
the same choice inside the C library (``sn_gpu_autotune``).

A block shape changes the order in which sites are updated (every shape is
an exact Metropolis sweep, so the physics is the same but trajectories
differ); the tuned shape is a per-lattice-size choice a run keeps fixed.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Sequence

from ._abi import check, lib
from .sim import ModelParams, Replica, Simulation, plan_candidates


def _mixed(params: ModelParams) -> bool:
    return len({float(d) for d in params.dipoles if float(d) > 0.0}) > 1


def tune(params: ModelParams, replica: Replica, max_candidates: int = 6, sweeps: int = 5,
         warmup: int = 2) -> tuple:
    """(best (bx, by, bz), [(shape, ms per sweep), ...]) for one lattice size."""
    cands = plan_candidates(replica.X, replica.Y, replica.Z, params.cutoff, _mixed(params), max_candidates)
    results = []
    for c in cands:
        shape = (c["bx"], c["by"], c["bz"])
        rep = dataclasses.replace(replica, block=shape)
        with Simulation(params, [rep]) as sim:
            sim.init_lattice(0)
            sim.set_recompute(0)
            sim.sweep(warmup)
            _, ms, _ = sim.phase_times(sweeps)
        results.append((shape, ms))
    best = min(results, key=lambda r: r[1])[0]
    return best, results


def _build_id() -> str:
    """The GPU and the library build a tuned shape was measured on: a shape
    tuned on another device or an older kernel is not reused."""
    import hashlib
    import os
    from ._abi import library_path
    gpu = "cpu"
    try:
        import torch
        if torch.cuda.is_available():
            gpu = torch.cuda.get_device_name().replace(" ", "_")
    except Exception:
        pass
    h = hashlib.sha1()
    try:
        with open(library_path(), "rb") as f:
            h.update(f.read())
    except OSError:
        h.update(b"unbuilt")
    return "%s/%s" % (gpu, h.hexdigest()[:12])


def _cache_key(params: ModelParams, r: Replica) -> str:
    return "%s/%dx%dx%d/rc%d/%s/%s" % (_build_id(), r.X, r.Y, r.Z, int(params.cutoff),
                                      "mixed" if _mixed(params) else "uniform", params.sweep_method)


def tune_table(params: ModelParams, replicas: Sequence[Replica], cache: str | None = None, **kw) -> list:
    """The table with each replica's block shape tuned (once per distinct size).

    cache: a JSON file of earlier choices (GPU and library build, lattice
    size, cutoff, mixed or uniform lengths, sweep method -> block shape);
    sizes found there are not timed again, new choices are added to it."""
    import json
    import os
    known = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            known = {k: tuple(v) for k, v in json.load(f).items()}
    chosen = {}
    out = []
    for r in replicas:
        key = _cache_key(params, r)
        if key not in chosen:
            chosen[key] = known[key] if key in known else tune(params, r, **kw)[0]
        out.append(dataclasses.replace(r, block=chosen[key]))
    if cache and any(k not in known for k in chosen):
        known.update(chosen)
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump({k: list(v) for k, v in sorted(known.items())}, f, indent=1)
        os.replace(tmp, cache)
    return out


def tune_native(params: ModelParams, replica: Replica, max_candidates: int = 6, sweeps: int = 5) -> tuple:
    """The same choice made inside the C ABI (``sn_gpu_autotune``, what a C host
    calls): ((bx, by, bz), ms per sweep of that shape)."""
    blk = (ctypes.c_int * 3)()
    ms = ctypes.c_double(0.0)
    cp, d = params.to_c(), replica.to_c()
    check(lib().sn_gpu_autotune(ctypes.byref(cp), ctypes.byref(d), int(max_candidates), int(sweeps), blk,
                                ctypes.byref(ms)))
    return (blk[0], blk[1], blk[2]), ms.value
