"""Python host API over the C ABI (``include/sn_gpu.h``).

``Simulation`` owns one handle: a replica table of dipole lattices resident
in HBM.  The reference keeps the same state in globals and drives it from
``main()`` (src/starrynight-main.c:125-277); the method names below follow
that driver's steps: initialise the lattice, run Monte Carlo sweeps
(``MC_moves``), read observables between megasteps.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi
from ._abi import SnError, check, lib

_f64p = ctypes.POINTER(ctypes.c_double)


def _ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


@dataclass
class ModelParams:
    """The starrynight.cfg keys of the hot path (src/starrynight-config.c:123-166)."""

    cutoff: int = 3                   # DipoleCutOff
    cage_strain: float = 1.0          # CageStrain
    K: float = 0.0                    # K (used only when > 0)
    efield: Sequence[float] = (0.0, 0.0, 0.0)
    dipoles: Sequence[float] = (1.0,)     # Dipoles
    prevalence: Sequence[float] = (1.0,)  # Prevalence
    constrain_to_x: bool = False      # ConstrainToX
    dim: int = 3
    seed: int = 1
    # "auto", "stencil" (sum the cutoff stencil per move) or "cached"
    # (incremental local fields); see SN_SWEEP_* in include/sn_gpu.h
    sweep_method: str = "auto"

    def to_c(self) -> _abi.Params:
        if len(self.dipoles) != len(self.prevalence):
            raise ValueError("Dipoles and Prevalence must have the same length")
        if not 1 <= len(self.dipoles) <= _abi.SN_MAX_SPECIES:
            raise ValueError("1..%d species" % _abi.SN_MAX_SPECIES)
        p = _abi.Params()
        p.cutoff, p.dim, p.constrain_to_x = int(self.cutoff), int(self.dim), int(bool(self.constrain_to_x))
        p.cage_strain, p.K = float(self.cage_strain), float(self.K)
        for k in range(3):
            p.efield[k] = float(self.efield[k])
        p.n_species = len(self.dipoles)
        for i, (d, q) in enumerate(zip(self.dipoles, self.prevalence)):
            p.dipoles[i], p.prevalence[i] = float(d), float(q)
        p.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        if self.sweep_method not in _abi.SWEEP_METHODS:
            raise ValueError("sweep_method must be one of %s" % sorted(_abi.SWEEP_METHODS))
        p.sweep_method = _abi.SWEEP_METHODS[self.sweep_method]
        return p


@dataclass
class Replica:
    X: int
    Y: int
    Z: int
    T: float = 300.0
    efield: Sequence[float] | None = None
    seed: int = 0
    block: Sequence[int] | None = None  # forced block shape (bx, by, bz); None: the planner's choice

    def to_c(self) -> _abi.ReplicaDesc:
        d = _abi.ReplicaDesc()
        d.X, d.Y, d.Z, d.T = int(self.X), int(self.Y), int(self.Z), float(self.T)
        if self.efield is not None:
            d.has_efield = 1
            for k in range(3):
                d.efield[k] = float(self.efield[k])
        d.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        if self.block is not None:
            for k in range(3):
                d.block[k] = int(self.block[k])
        return d

    @property
    def n_sites(self) -> int:
        return self.X * self.Y * self.Z


def plan_schedule(X: int, Y: int, Z: int, cutoff: int, mixed: bool = False) -> dict:
    info = _abi.ScheduleInfo()
    check(lib().sn_plan_schedule(X, Y, Z, cutoff, int(mixed), ctypes.byref(info)))
    return info.as_dict()


def plan_candidates(X: int, Y: int, Z: int, cutoff: int, mixed: bool = False, max_out: int = 8) -> list:
    """Feasible schedules in the planner's preference order (host-only)."""
    arr = (_abi.ScheduleInfo * max_out)()
    n = ctypes.c_int(0)
    check(lib().sn_plan_candidates(X, Y, Z, cutoff, int(mixed), arr, max_out, ctypes.byref(n)))
    return [arr[i].as_dict() for i in range(n.value)]


def check_schedule(X: int, Y: int, Z: int, cutoff: int, sched: dict) -> bool:
    info = _abi.ScheduleInfo(**{k: int(v) for k, v in sched.items()})
    return bool(lib().sn_check_schedule(X, Y, Z, cutoff, ctypes.byref(info)))


def check_flow(params: "ModelParams", replicas: Sequence["Replica"]) -> dict:
    """Host-only verification of the dataflow schedule of a replica table (raises on a defect)."""
    cp = params.to_c()
    arr = (_abi.ReplicaDesc * len(replicas))(*[r.to_c() for r in replicas])
    st = np.zeros(3, np.uint64)
    check(lib().sn_check_flow(ctypes.byref(cp), len(replicas), arr, _ptr(st)))
    return {"blocks": int(st[0]), "dependencies": int(st[1]), "max_dependencies": int(st[2])}


def fp32_peak():
    """(measured FP32 TFLOP/s on the current device, nominal max SM clock MHz)."""
    t, c = ctypes.c_double(0.0), ctypes.c_double(0.0)
    check(lib().sn_gpu_fp32_peak(ctypes.byref(t), ctypes.byref(c)))
    return t.value, c.value


def neighbour_count(cutoff: int, Z: int) -> int:
    return lib().sn_neighbour_count(cutoff, Z)


def philox(ctr: np.ndarray, key: np.ndarray) -> np.ndarray:
    """Philox4x32-10 on the device; ctr (n,4) uint32, key (n,2) uint32."""
    ctr = np.ascontiguousarray(ctr, np.uint32)
    key = np.ascontiguousarray(key, np.uint32)
    out = np.zeros_like(ctr)
    check(lib().sn_gpu_philox(_ptr(ctr), _ptr(key), _ptr(out), ctr.shape[0]))
    return out


class Simulation:
    """A replica table of dipole lattices on the GPU."""

    def __init__(self, params: ModelParams, replicas: Sequence[Replica]):
        self.params = params
        self.replicas = list(replicas)
        cp = params.to_c()
        arr = (_abi.ReplicaDesc * len(self.replicas))(*[r.to_c() for r in self.replicas])
        h = ctypes.c_void_p()
        check(lib().sn_gpu_init(ctypes.byref(cp), len(self.replicas), arr, ctypes.byref(h)))
        self._h = h

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sn_gpu_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status: int) -> None:
        check(status, self._h)

    def n_sites(self, replica: int = 0) -> int:
        return self.replicas[replica].n_sites

    # -- lattice ---------------------------------------------------------------
    def init_lattice(self, replica: int = 0, pattern: str = "random", seed: int = 0) -> None:
        pat = {"random": _abi.SN_LATTICE_RANDOM, "ferroelectric": _abi.SN_LATTICE_FERROELECTRIC}[pattern]
        self._ck(lib().sn_gpu_init_lattice(self._h, replica, pat, int(seed)))

    def upload(self, replica: int, xyz: np.ndarray, length: np.ndarray | None = None) -> None:
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1)
        n = self.n_sites(replica)
        if xyz.size != 3 * n:
            raise ValueError("xyz must hold 3*%d floats" % n)
        ln = None
        if length is not None:
            ln = np.ascontiguousarray(length, np.float32).reshape(-1)
            if ln.size != n:
                raise ValueError("length must hold %d floats" % n)
        self._ck(lib().sn_gpu_upload_lattice(self._h, replica, _ptr(xyz), _ptr(ln)))

    def upload_ptr(self, replica: int, xyz_ptr: int, len_ptr: int | None = None) -> None:
        """Upload from raw host pointers (e.g. pinned buffers)."""
        self._ck(lib().sn_gpu_upload_lattice(self._h, replica, ctypes.c_void_p(xyz_ptr),
                                             ctypes.c_void_p(len_ptr) if len_ptr else None))

    def download(self, replica: int = 0):
        n = self.n_sites(replica)
        xyz = np.zeros((n, 3), np.float32)
        ln = np.zeros(n, np.float32)
        self._ck(lib().sn_gpu_download_lattice(self._h, replica, _ptr(xyz), _ptr(ln)))
        return xyz, ln

    def download_ptr(self, replica: int, xyz_ptr: int, len_ptr: int | None = None) -> None:
        self._ck(lib().sn_gpu_download_lattice(self._h, replica, ctypes.c_void_p(xyz_ptr),
                                               ctypes.c_void_p(len_ptr) if len_ptr else None))

    # -- Monte Carlo -------------------------------------------------------------
    def sweep(self, n: int = 1, counts: bool = False):
        """n sweeps of every replica; with counts, returns (accepted, rejected)."""
        if counts:
            a, r = ctypes.c_uint64(0), ctypes.c_uint64(0)
            self._ck(lib().sn_gpu_sweep(self._h, int(n), ctypes.byref(a), ctypes.byref(r)))
            return a.value, r.value
        self._ck(lib().sn_gpu_sweep(self._h, int(n), None, None))
        return None

    def sweep_download(self, n: int, outs, counts: bool = False):
        """n sweeps, then each replica's lattice into outs[r] (numpy (N, 3) float32,
        a raw pointer, or None to skip).  Pinned buffers are written by the last
        sweep itself; others by the staged download."""
        if len(outs) != len(self.replicas):
            raise ValueError("one output per replica")
        tab = (ctypes.c_void_p * len(outs))()
        keep = []
        for r, o in enumerate(outs):
            if o is None:
                continue
            if isinstance(o, int):
                tab[r] = o
            else:
                if not (isinstance(o, np.ndarray) and o.dtype == np.float32 and o.flags.c_contiguous
                        and o.size == 3 * self.n_sites(r)):
                    raise ValueError("replica %d: need a C-contiguous float32 array of %d values" % (r, 3 * self.n_sites(r)))
                keep.append(o)
                tab[r] = o.ctypes.data
        a, j = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._ck(lib().sn_gpu_sweep_download(self._h, int(n), tab, ctypes.byref(a) if counts else None,
                                             ctypes.byref(j) if counts else None))
        return (a.value, j.value) if counts else None

    def sweep_count(self) -> int:
        v = ctypes.c_uint64(0)
        self._ck(lib().sn_gpu_sweep_count(self._h, ctypes.byref(v)))
        return v.value

    def set_sweep_count(self, sweeps: int) -> None:
        """Restore the sweep counter that keys the random stream (resume from a checkpoint)."""
        self._ck(lib().sn_gpu_set_sweep_count(self._h, int(sweeps)))

    # -- analysis (src/starrynight-analysis.c) ------------------------------------
    def potential(self, replica: int = 0, cutoff: int = 6) -> np.ndarray:
        """dipole_potential at every site (FP64, bit-equal to the reference)."""
        out = np.zeros(self.n_sites(replica), np.float64)
        self._ck(lib().sn_gpu_potential(self._h, replica, int(cutoff), _ptr(out)))
        return out

    def efield(self, replica: int = 0, cutoff: int = 4, half_offset: bool = False) -> np.ndarray:
        """|E| of dipole_electricfield (or dipole_electricfieldoffset) at every site."""
        out = np.zeros(self.n_sites(replica), np.float64)
        self._ck(lib().sn_gpu_efield(self._h, replica, int(cutoff), int(bool(half_offset)), _ptr(out)))
        return out

    def radial_order(self, replica: int = 0, cutoff: int = 9):
        """(fe_sum, afe_sum, count) per |r|^2 bin of radial_order_parameter (FP64 sums)."""
        nb = cutoff * cutoff + 1
        fe, afe, cnt = np.zeros(nb), np.zeros(nb), np.zeros(nb, np.int64)
        self._ck(lib().sn_gpu_radial_order(self._h, replica, int(cutoff), _ptr(fe), _ptr(afe), _ptr(cnt)))
        return fe, afe, cnt

    def order_parameters(self, replica: int = 0):
        """(polarisation() = sum p_x / N, landau_order() = |sum p|^2, sum p) -- unweighted."""
        pol, lan, s3 = ctypes.c_double(0.0), ctypes.c_double(0.0), np.zeros(3)
        self._ck(lib().sn_gpu_order_parameters(self._h, replica, ctypes.byref(pol), ctypes.byref(lan), _ptr(s3)))
        return pol.value, lan.value, s3

    # -- energies / observables -----------------------------------------------------
    def energy(self, replica: int = 0, precision: str = "fp32", site: bool = False):
        prec = _abi.SN_ENERGY_FP64 if precision == "fp64" else _abi.SN_ENERGY_FP32
        E = ctypes.c_double(0.0)
        se = np.zeros(self.n_sites(replica), np.float64) if site else None
        self._ck(lib().sn_gpu_energy(self._h, replica, prec, ctypes.byref(E), _ptr(se)))
        return (E.value, se) if site else E.value

    def observables(self) -> dict:
        n = len(self.replicas)
        e, p, v = np.zeros(n), np.zeros(n), np.zeros((n, 3))
        self._ck(lib().sn_gpu_observables(self._h, _ptr(e), _ptr(p), _ptr(v)))
        return {"E_per_site": e, "P_abs": p, "P_vec": v}

    def history(self, replica: int = 0, max_entries: int = 4096):
        e, p = np.zeros(max_entries), np.zeros(max_entries)
        n = ctypes.c_int(0)
        self._ck(lib().sn_gpu_history(self._h, replica, max_entries, _ptr(e), _ptr(p), ctypes.byref(n)))
        return e[: n.value].copy(), p[: n.value].copy()

    def recompute(self, precision: str = "fp32") -> float:
        prec = _abi.SN_ENERGY_FP64 if precision == "fp64" else _abi.SN_ENERGY_FP32
        d = ctypes.c_double(0.0)
        self._ck(lib().sn_gpu_recompute(self._h, prec, ctypes.byref(d)))
        return d.value

    def set_recompute(self, every: int, precision: str = "fp32") -> None:
        prec = _abi.SN_ENERGY_FP64 if precision == "fp64" else _abi.SN_ENERGY_FP32
        self._ck(lib().sn_gpu_set_recompute(self._h, int(every), prec))

    def drift(self):
        d, n = ctypes.c_double(0.0), ctypes.c_int(0)
        self._ck(lib().sn_gpu_drift(self._h, ctypes.byref(d), ctypes.byref(n)))
        return d.value, n.value

    # -- run control ------------------------------------------------------------------
    def set_field(self, replica: int, efield: Sequence[float]) -> None:
        arr = (ctypes.c_float * 3)(*[float(v) for v in efield])
        self._ck(lib().sn_gpu_set_field(self._h, replica, arr))

    def set_temperature(self, replica: int, T: float) -> None:
        self._ck(lib().sn_gpu_set_temperature(self._h, replica, float(T)))

    def temperature(self, replica: int) -> float:
        t = ctypes.c_float(0.0)
        self._ck(lib().sn_gpu_get_temperature(self._h, replica, ctypes.byref(t)))
        return t.value

    def set_exchange(self, every: int) -> None:
        self._ck(lib().sn_gpu_set_exchange(self._h, int(every)))

    def exchange_stats(self):
        a, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._ck(lib().sn_gpu_exchange_stats(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # -- differentiation ------------------------------------------------------------------
    def adjoint(self, replica: int = 0, grad: bool = True):
        """(dE/dp (N,3) float32 or None, dE/d(Dipole, CageStrain, Ex, Ey, Ez), E)."""
        g = np.zeros((self.n_sites(replica), 3), np.float32) if grad else None
        dp = np.zeros(5, np.float64)
        E = ctypes.c_double(0.0)
        self._ck(lib().sn_gpu_adjoint(self._h, replica, _ptr(g), _ptr(dp), ctypes.byref(E)))
        return g, dp, E.value

    def quench(self, replica: int, n_steps: int, step: float) -> np.ndarray:
        tr = np.zeros(n_steps + 1)
        self._ck(lib().sn_gpu_quench(self._h, replica, int(n_steps), float(step), _ptr(tr)))
        return tr

    # -- introspection -------------------------------------------------------------------------
    def schedule(self, replica: int = 0) -> dict:
        info = _abi.ScheduleInfo()
        self._ck(lib().sn_gpu_schedule(self._h, replica, ctypes.byref(info)))
        return info.as_dict()

    def launches(self) -> int:
        v = ctypes.c_uint64(0)
        self._ck(lib().sn_gpu_launch_count(self._h, ctypes.byref(v)))
        return v.value

    def stream_ptr(self) -> int:
        return lib().sn_gpu_stream(self._h) or 0

    def phase_times(self, n_sweeps: int = 3):
        """(mean ms of one block-colour launch, mean ms per sweep, launches per sweep)."""
        a, b, n = ctypes.c_double(0.0), ctypes.c_double(0.0), ctypes.c_int(0)
        self._ck(lib().sn_gpu_phase_times(self._h, int(n_sweeps), ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)))
        return a.value, b.value, n.value

    def sweep_timed(self, n: int) -> float:
        """n sweeps; returns their device time in ms (CUDA events on the handle's stream)."""
        ms = ctypes.c_double(0.0)
        self._ck(lib().sn_gpu_sweep_timed(self._h, int(n), ctypes.byref(ms)))
        return ms.value

    def set_wait_limit(self, polls: int) -> None:
        """Polls of one dependency flag before a dataflow block reports SN_ERR_TIMEOUT."""
        self._ck(lib().sn_gpu_set_wait_limit(self._h, int(polls)))

    def field_cache_check(self, replica: int = 0) -> int:
        """Entries of the cached-field sweep's cache that differ from a fresh field pass (0 = exact)."""
        v = ctypes.c_uint64(0)
        self._ck(lib().sn_gpu_field_cache_check(self._h, replica, ctypes.byref(v)))
        return v.value

    def test_stall_block(self, item: int) -> None:
        """Test hook: dataflow item `item` waits on a flag nobody sets (-1 restores)."""
        self._ck(lib().sn_gpu_test_stall_block(self._h, int(item)))

    def flow_stats(self) -> dict:
        """Dataflow schedule statistics since the last call (see sn_gpu_flow_stats)."""
        s = np.zeros(4, np.uint64)
        self._ck(lib().sn_gpu_flow_stats(self._h, _ptr(s)))
        return {"dataflow": bool(s[0]), "grid": int(s[1]), "waited_blocks": int(s[2]), "polls": int(s[3])}

    def proposals(self, replica: int, sites: np.ndarray, sweep: int) -> np.ndarray:
        sites = np.ascontiguousarray(sites, np.uint32)
        out = np.zeros((sites.size, 4), np.float32)
        self._ck(lib().sn_gpu_proposals(self._h, replica, _ptr(sites), sites.size, int(sweep), _ptr(out)))
        return out
