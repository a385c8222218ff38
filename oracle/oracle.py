"""ctypes wrapper of the CPU oracle (``oracle/libsn_oracle.so``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``.  The product package never imports
this module.

The C library restates the reference hot path (see ``sn_oracle.h`` for the
file:line each function follows) and mirrors the GPU colour schedule with an
FP64 energy change.  ``ref_harness`` (built into ``oracle/_ref/`` from the
reference tree) wraps the unmodified reference sources; it exists only where
the reference tree is present.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(ref: bool = False) -> None:
    """Compile the oracle (and, with ``ref``, the reference harness)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "libsn_oracle.so")
        src = os.path.join(HERE, "sn_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = ctypes.CDLL(path)
        _declare(_LIB)
        _declare_analysis(_LIB)
    return _LIB


class Model(ctypes.Structure):
    _fields_ = [
        ("X", ctypes.c_int), ("Y", ctypes.c_int), ("Z", ctypes.c_int),
        ("cutoff", ctypes.c_int), ("dim", ctypes.c_int), ("constrain_to_x", ctypes.c_int),
        ("beta", ctypes.c_double), ("efield", ctypes.c_float * 3),
        ("K", ctypes.c_double), ("cage_strain", ctypes.c_double),
    ]


class Schedule(ctypes.Structure):
    _fields_ = [
        ("bx", ctypes.c_int), ("by", ctypes.c_int), ("bz", ctypes.c_int),
        ("nbx", ctypes.c_int), ("nby", ctypes.c_int), ("nbz", ctypes.c_int),
        ("mx", ctypes.c_int), ("my", ctypes.c_int), ("mz", ctypes.c_int),
        ("s", ctypes.c_int), ("merge", ctypes.c_int),
    ]


class Stream(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("beta", ctypes.c_float), ("length", ctypes.c_float)]


class MT(ctypes.Structure):
    _fields_ = [("mt", ctypes.c_uint32 * 624), ("mti", ctypes.c_int32)]


_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u32 = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_P = ctypes.POINTER


def _declare(L: ctypes.CDLL) -> None:
    L.sno_mt_seed.argtypes = [_P(MT), ctypes.c_uint32]
    L.sno_mt_u32.argtypes = [_P(MT)]
    L.sno_mt_u32.restype = ctypes.c_uint32
    L.sno_mt_real1.argtypes = [_P(MT)]
    L.sno_mt_real1.restype = ctypes.c_double
    L.sno_mt_real2.argtypes = [_P(MT)]
    L.sno_mt_real2.restype = ctypes.c_double
    L.sno_philox4x32_10.argtypes = [_u32, _u32, _u32]
    L.sno_gen_neighbours.argtypes = [ctypes.c_int, ctypes.c_int, _i, _i, _i, _f, ctypes.c_int]
    L.sno_gen_neighbours.restype = ctypes.c_int
    L.sno_ref_init_random.argtypes = [_P(Model), _f, _P(MT), ctypes.c_int, _f, _f]
    L.sno_ref_site_energy.argtypes = [_P(Model), _f, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f, _f]
    L.sno_ref_site_energy.restype = ctypes.c_double
    L.sno_ref_mc_moves.argtypes = [_P(Model), _f, _P(MT), ctypes.c_longlong,
                                   _P(ctypes.c_uint64), _P(ctypes.c_uint64)]
    L.sno_colour_sweep.argtypes = [_P(Model), _P(Schedule), _P(Stream), ctypes.c_uint32,
                                   _f, _f, _f, _f, _vp, ctypes.c_double,
                                   _P(ctypes.c_uint64), _P(ctypes.c_uint64), _P(ctypes.c_double),
                                   _vp, _vp]
    L.sno_colour_sweep.restype = ctypes.c_uint64
    L.sno_proposal.argtypes = [_P(Model), _P(Stream), ctypes.c_uint32, ctypes.c_uint32, _f, _f]
    L.sno_energy64.argtypes = [_P(Model), _f, _f, _f, _f, ctypes.c_double, _vp, _vp, _vp,
                               _P(ctypes.c_double)]
    L.sno_energy64.restype = ctypes.c_double
    L.sno_delta_energy64.argtypes = [_P(Model), _f, _f, _f, _f, ctypes.c_int, _f]
    L.sno_delta_energy64.restype = ctypes.c_double


def _declare_analysis(L: ctypes.CDLL) -> None:
    L.sno_potential_map.argtypes = [_f, _f, _f, _f] + [ctypes.c_int] * 4 + [_d]
    L.sno_efield_map.argtypes = [_f, _f, _f] + [ctypes.c_int] * 5 + [_d]
    L.sno_radial_order.argtypes = [_f, _f, _f] + [ctypes.c_int] * 5 + [_d, _d, _i64]
    L.sno_order_params.argtypes = [_f, _f, _f, ctypes.c_longlong, _P(ctypes.c_double), _P(ctypes.c_double), _d]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def make_model(X, Y, Z, cutoff, T=300.0, efield=(0.0, 0.0, 0.0), K=0.0, cage_strain=1.0,
               constrain_to_x=False, dim=3, beta=None) -> Model:
    """A model with the reference's beta = 1/((float)T/300) (src/starrynight-main.c:215)."""
    if beta is None:
        beta = ref_beta(T) if isinstance(T, int) else 300.0 / float(T)
    m = Model()
    m.X, m.Y, m.Z = X, Y, Z
    m.cutoff, m.dim, m.constrain_to_x = cutoff, dim, int(bool(constrain_to_x))
    m.beta = beta
    for k in range(3):
        m.efield[k] = efield[k]
    m.K, m.cage_strain = K, cage_strain
    return m


def ref_beta(T: int) -> float:
    """beta exactly as the reference computes it: 1/((float)T/300.0)."""
    return 1.0 / (float(np.float32(T)) / 300.0)


class MTState:
    def __init__(self, seed: int):
        self.s = MT()
        lib().sno_mt_seed(ctypes.byref(self.s), ctypes.c_uint32(seed & 0xFFFFFFFF))

    def u32(self) -> int:
        return lib().sno_mt_u32(ctypes.byref(self.s))

    def real1(self) -> float:
        return lib().sno_mt_real1(ctypes.byref(self.s))

    def real2(self) -> float:
        return lib().sno_mt_real2(ctypes.byref(self.s))


def philox(ctr, key) -> np.ndarray:
    out = np.zeros(4, np.uint32)
    lib().sno_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def neighbours(cutoff: int, Z: int):
    side = 2 * cutoff + 1
    mx = side ** 3
    dx, dy, dz = (np.zeros(mx, np.int32) for _ in range(3))
    d = np.zeros(mx, np.float32)
    n = lib().sno_gen_neighbours(cutoff, Z, dx, dy, dz, d, mx)
    return np.stack([dx[:n], dy[:n], dz[:n]], axis=1), d[:n]


def ref_init_random(m: Model, mt: MTState, lengths=(1.0,), prevalence=(1.0,)) -> np.ndarray:
    lat = np.zeros((m.X * m.Y * m.Z, 4), np.float32)
    lib().sno_ref_init_random(ctypes.byref(m), lat.reshape(-1), ctypes.byref(mt.s), len(lengths),
                              np.asarray(lengths, np.float32), np.asarray(prevalence, np.float32))
    return lat


def ref_mc_moves(m: Model, lat4: np.ndarray, mt: MTState, moves: int):
    a, r = ctypes.c_uint64(0), ctypes.c_uint64(0)
    lib().sno_ref_mc_moves(ctypes.byref(m), lat4.reshape(-1), ctypes.byref(mt.s), int(moves),
                           ctypes.byref(a), ctypes.byref(r))
    return a.value, r.value


def ref_site_energy(m: Model, lat4: np.ndarray, x: int, y: int, z: int, new4) -> float:
    i = (x * m.Y + y) * m.Z + z
    return lib().sno_ref_site_energy(ctypes.byref(m), lat4.reshape(-1), x, y, z,
                                     np.asarray(new4, np.float32), np.ascontiguousarray(lat4[i]))


def make_schedule(d: dict) -> Schedule:
    s = Schedule()
    for k in ("bx", "by", "bz", "nbx", "nby", "nbz", "mx", "my", "mz", "s", "merge"):
        setattr(s, k, int(d.get(k, 0)))
    return s


def make_stream(seed: int, beta: float, length: float = 1.0) -> Stream:
    st = Stream()
    st.seed, st.beta, st.length = seed, beta, length
    return st


@dataclass
class SweepResult:
    accepted: int
    borderline: int
    hard: int
    dE_sum: float
    margin: np.ndarray | None
    accept: np.ndarray | None


def colour_sweep(m: Model, sched: Schedule, st: Stream, sweep: int, px, py, pz, length,
                 gpu_after=None, tol: float = 0.0, record: bool = False) -> SweepResult:
    """One sweep in the GPU order; px/py/pz are updated in place (float32)."""
    N = m.X * m.Y * m.Z
    nb, nh, de = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_double(0.0)
    ga = None
    if gpu_after is not None:
        ga = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float32).reshape(-1) for a in gpu_after]))
    margin = np.zeros(N, np.float64) if record else None
    acc = np.zeros(N, np.uint8) if record else None
    n = lib().sno_colour_sweep(ctypes.byref(m), ctypes.byref(sched), ctypes.byref(st), sweep,
                               px, py, pz, length, _ptr(ga), tol, ctypes.byref(nb), ctypes.byref(nh),
                               ctypes.byref(de), _ptr(margin), _ptr(acc))
    return SweepResult(int(n), nb.value, nh.value, de.value, margin, acc)


def proposal(m: Model, st: Stream, site: int, sweep: int):
    p = np.zeros(3, np.float32)
    u = np.zeros(1, np.float32)
    lib().sno_proposal(ctypes.byref(m), ctypes.byref(st), site, sweep, p, u)
    return p, float(u[0])


def energy64(m: Model, px, py, pz, length, dipole: float = 1.0, site: bool = False, grad: bool = False):
    N = m.X * m.Y * m.Z
    se = np.zeros(N, np.float64) if site else None
    g = np.zeros(3 * N, np.float64) if grad else None
    dp = np.zeros(5, np.float64)
    edd = ctypes.c_double(0.0)
    E = lib().sno_energy64(ctypes.byref(m), px, py, pz, length, dipole, _ptr(se), _ptr(g), _ptr(dp),
                           ctypes.byref(edd))
    return {"E": E, "site": se, "grad": None if g is None else g.reshape(N, 3), "dparams": dp,
            "E_dd": edd.value}


def delta_energy64(m: Model, px, py, pz, length, site: int, newp) -> float:
    return lib().sno_delta_energy64(ctypes.byref(m), px, py, pz, length, site, np.asarray(newp, np.float32))


def soa(lat4: np.ndarray):
    """AoS (x,y,z,len) -> four contiguous float32 arrays."""
    return tuple(np.ascontiguousarray(lat4[:, k]) for k in range(4))


# ---- analysis (src/starrynight-analysis.c) ----

def _soa3(px, py, pz):
    return [np.ascontiguousarray(a, np.float32).reshape(-1) for a in (px, py, pz)]


def potential_map(px, py, pz, length, shape, cutoff: int = 6) -> np.ndarray:
    """dipole_potential at every site (bit-equal to the reference)."""
    X, Y, Z = shape
    out = np.zeros(X * Y * Z, np.float64)
    a = _soa3(px, py, pz)
    lib().sno_potential_map(*a, np.ascontiguousarray(length, np.float32).reshape(-1), X, Y, Z, int(cutoff), out)
    return out


def efield_map(px, py, pz, shape, cutoff: int = 4, half: bool = False) -> np.ndarray:
    """|E| of dipole_electricfield (half=False) or dipole_electricfieldoffset (half=True)."""
    X, Y, Z = shape
    out = np.zeros(X * Y * Z, np.float64)
    lib().sno_efield_map(*_soa3(px, py, pz), X, Y, Z, int(cutoff), int(bool(half)), out)
    return out


def radial_order(px, py, pz, shape, cutoff: int = 9, float_sums: bool = False):
    """(fe_sum, afe_sum, count) per |r|^2 bin of radial_order_parameter: FP64 sums, or the
    reference's own float sums with float_sums=True."""
    X, Y, Z = shape
    nb = cutoff * cutoff + 1
    fe, afe, cnt = np.zeros(nb), np.zeros(nb), np.zeros(nb, np.int64)
    lib().sno_radial_order(*_soa3(px, py, pz), X, Y, Z, int(cutoff), int(bool(float_sums)), fe, afe, cnt)
    return fe, afe, cnt


def order_params(px, py, pz):
    """(polarisation_x, landau, orientation sum[3]) of polarisation() / landau_order()."""
    a = _soa3(px, py, pz)
    pol, lan, s3 = ctypes.c_double(0.0), ctypes.c_double(0.0), np.zeros(3)
    lib().sno_order_params(*a, a[0].size, ctypes.byref(pol), ctypes.byref(lan), s3)
    return pol.value, lan.value, s3
