"""ctypes declarations of the C ABI in ``include/sn_gpu.h``.

The shared library is built in-tree (``starrynight_gb300/lib/libsn_gpu.so``);
importing the package never falls back to anything else: a missing library
raises.
"""
from __future__ import annotations

import ctypes
import os

from . import native as _build

SN_MAX_SPECIES = 10
SN_MAX_CUTOFF = 6
SN_LATTICE_RANDOM = 0
SN_LATTICE_FERROELECTRIC = 1
SN_ENERGY_FP32 = 0
SN_ENERGY_FP64 = 1

STATUS = {
    0: "SN_OK", 1: "SN_ERR_ARG", 2: "SN_ERR_CONFIG", 3: "SN_ERR_SCHEDULE", 4: "SN_ERR_CUDA",
    5: "SN_ERR_NOMEM", 6: "SN_ERR_TIMEOUT", 7: "SN_ERR_UNSUPPORTED",
}


class SnError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (STATUS.get(status, str(status)), message))
        self.status = status
        self.name = STATUS.get(status, str(status))


SN_SWEEP_AUTO, SN_SWEEP_STENCIL, SN_SWEEP_CACHED = 0, 1, 2
SWEEP_METHODS = {"auto": SN_SWEEP_AUTO, "stencil": SN_SWEEP_STENCIL, "cached": SN_SWEEP_CACHED}


class Params(ctypes.Structure):
    _fields_ = [
        ("cutoff", ctypes.c_int), ("dim", ctypes.c_int), ("constrain_to_x", ctypes.c_int),
        ("cage_strain", ctypes.c_double), ("K", ctypes.c_double), ("efield", ctypes.c_float * 3),
        ("n_species", ctypes.c_int), ("dipoles", ctypes.c_float * SN_MAX_SPECIES),
        ("prevalence", ctypes.c_float * SN_MAX_SPECIES), ("seed", ctypes.c_uint64), ("sweep_method", ctypes.c_int),
    ]


class ReplicaDesc(ctypes.Structure):
    _fields_ = [
        ("X", ctypes.c_int), ("Y", ctypes.c_int), ("Z", ctypes.c_int), ("T", ctypes.c_float),
        ("has_efield", ctypes.c_int), ("efield", ctypes.c_float * 3), ("seed", ctypes.c_uint64),
        ("block", ctypes.c_int * 3),
    ]


class ScheduleInfo(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in ("bx", "by", "bz", "nbx", "nby", "nbz", "mx", "my", "mz", "s",
                                             "halo", "tile_slots", "smem_bytes", "merge", "threads",
                                             "field_cache")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB = None
_vp = ctypes.c_void_p
_i = ctypes.c_int
_P = ctypes.POINTER


def library_path() -> str:
    # SN_GPU_LIB selects another build of the same library (tuning builds)
    return os.environ.get("SN_GPU_LIB") or _build.lib_path()


def lib() -> ctypes.CDLL:
    """Load the CUDA library.  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError("libsn_gpu.so is not built (run starrynight_gb300.build.build()); "
                               "there is no CPU fallback")
        L = ctypes.CDLL(path)
        h = _vp
        sig = {
            "sn_gpu_init": ([_P(Params), _i, _P(ReplicaDesc), _P(h)], _i),
            "sn_gpu_destroy": ([h], _i),
            "sn_gpu_status_string": ([_i], ctypes.c_char_p),
            "sn_gpu_last_error": ([h], ctypes.c_char_p),
            "sn_gpu_host_alloc": ([ctypes.c_size_t], _vp),
            "sn_gpu_host_free": ([_vp], None),
            "sn_gpu_init_lattice": ([h, _i, _i, ctypes.c_uint64], _i),
            "sn_gpu_upload_lattice": ([h, _i, _vp, _vp], _i),
            "sn_gpu_download_lattice": ([h, _i, _vp, _vp], _i),
            "sn_gpu_sweep": ([h, _i, _P(ctypes.c_uint64), _P(ctypes.c_uint64)], _i),
            "sn_gpu_sweep_download": ([h, _i, _P(ctypes.c_void_p), _P(ctypes.c_uint64), _P(ctypes.c_uint64)], _i),
            "sn_gpu_sweep_count": ([h, _P(ctypes.c_uint64)], _i),
            "sn_gpu_set_sweep_count": ([h, ctypes.c_uint64], _i),
            "sn_gpu_energy": ([h, _i, _i, _P(ctypes.c_double), _vp], _i),
            "sn_gpu_observables": ([h, _vp, _vp, _vp], _i),
            "sn_gpu_history": ([h, _i, _i, _vp, _vp, _P(_i)], _i),
            "sn_gpu_recompute": ([h, _i, _P(ctypes.c_double)], _i),
            "sn_gpu_set_recompute": ([h, _i, _i], _i),
            "sn_gpu_drift": ([h, _P(ctypes.c_double), _P(_i)], _i),
            "sn_gpu_set_field": ([h, _i, _P(ctypes.c_float)], _i),
            "sn_gpu_set_temperature": ([h, _i, ctypes.c_float], _i),
            "sn_gpu_get_temperature": ([h, _i, _P(ctypes.c_float)], _i),
            "sn_gpu_set_exchange": ([h, _i], _i),
            "sn_gpu_exchange_stats": ([h, _P(ctypes.c_uint64), _P(ctypes.c_uint64)], _i),
            "sn_gpu_adjoint": ([h, _i, _vp, _vp, _P(ctypes.c_double)], _i),
            "sn_gpu_quench": ([h, _i, _i, ctypes.c_float, _vp], _i),
            "sn_gpu_schedule": ([h, _i, _P(ScheduleInfo)], _i),
            "sn_plan_schedule": ([_i, _i, _i, _i, _i, _P(ScheduleInfo)], _i),
            "sn_plan_candidates": ([_i, _i, _i, _i, _i, _P(ScheduleInfo), _i, _P(_i)], _i),
            "sn_gpu_autotune": ([_P(Params), _P(ReplicaDesc), _i, _i, _P(_i), _P(ctypes.c_double)], _i),
            "sn_check_schedule": ([_i, _i, _i, _i, _P(ScheduleInfo)], _i),
            "sn_check_flow": ([_P(Params), _i, _P(ReplicaDesc), _vp], _i),
            "sn_gpu_launch_count": ([h, _P(ctypes.c_uint64)], _i),
            "sn_gpu_stream": ([h], _vp),
            "sn_neighbour_count": ([_i, _i], _i),
            "sn_gpu_philox": ([_vp, _vp, _vp, _i], _i),
            "sn_gpu_fp32_peak": ([_P(ctypes.c_double), _P(ctypes.c_double)], _i),
            "sn_gpu_energy_noalloc": ([_vp, _vp, _vp, _vp, _i, _i, _i, _P(Params), _vp, _P(ctypes.c_double), _vp], _i),
            "sn_gpu_phase_times": ([h, _i, _P(ctypes.c_double), _P(ctypes.c_double), _P(_i)], _i),
            "sn_gpu_proposals": ([h, _i, _vp, _i, ctypes.c_uint32, _vp], _i),
            "sn_gpu_potential": ([h, _i, _i, _vp], _i),
            "sn_gpu_flow_stats": ([h, _vp], _i),
            "sn_gpu_sweep_timed": ([h, _i, _P(ctypes.c_double)], _i),
            "sn_gpu_set_wait_limit": ([h, ctypes.c_uint32], _i),
            "sn_gpu_test_stall_block": ([h, _i], _i),
            "sn_gpu_field_cache_check": ([h, _i, _P(ctypes.c_uint64)], _i),
            "sn_gpu_efield": ([h, _i, _i, _i, _vp], _i),
            "sn_gpu_radial_order": ([h, _i, _i, _vp, _vp, _vp], _i),
            "sn_gpu_order_parameters": ([h, _i, _P(ctypes.c_double), _P(ctypes.c_double), _vp], _i),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def check(status: int, handle=None) -> None:
    if status != 0:
        msg = lib().sn_gpu_last_error(handle)
        raise SnError(status, msg.decode() if msg else "")


def exported_names() -> list:
    """Function names declared in include/sn_gpu.h."""
    import re
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "sn_gpu.h")
    src = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:sn_status|const char \*|int|void \*|void)\s*\*?\s*(sn_\w+)\s*\(", src, re.M)))
