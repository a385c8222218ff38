"""ctypes wrapper of ``oracle/_ref/libref_harness.so`` -- the unmodified
reference sources driven as a library.  TEST INFRASTRUCTURE ONLY.

Only available where the reference tree was present at build time (the
golden fixtures under ``tests/golden/`` are generated from it here and are
what the tests use elsewhere).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "_ref", "libref_harness.so")
_LIB = None

_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def available() -> bool:
    return os.path.exists(PATH)


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(PATH)
        L.refh_setup.argtypes = [ctypes.c_int] * 4 + [ctypes.c_double, ctypes.c_double, _f, ctypes.c_int,
                                                      ctypes.c_int, ctypes.c_int, _f, _f, ctypes.c_uint]
        L.refh_setup.restype = ctypes.c_int
        L.refh_get_lattice.argtypes = [_f]
        L.refh_set_lattice.argtypes = [_f]
        L.refh_mc_moves.argtypes = [ctypes.c_longlong]
        L.refh_counts.argtypes = [ctypes.POINTER(ctypes.c_ulonglong)] * 2
        L.refh_beta.restype = ctypes.c_double
        L.refh_site_energy.argtypes = [ctypes.c_int] * 3 + [_f]
        L.refh_site_energy.restype = ctypes.c_double
        L.refh_neighbours.argtypes = [_i, _f, ctypes.c_int]
        L.refh_neighbours.restype = ctypes.c_int
        L.refh_observables.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2
        L.refh_mt_next.restype = ctypes.c_uint
        L.refh_init_pattern.argtypes = [ctypes.c_char_p]
        L.refh_init_pattern.restype = ctypes.c_int
        L.refh_potential_map.argtypes = [_d]
        L.refh_efield_map.argtypes = [ctypes.c_int, ctypes.c_int, _d]
        L.refh_write.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.refh_write.restype = ctypes.c_int
        L.refh_capture.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.refh_capture.restype = ctypes.c_int
        _LIB = L
    return _LIB


class RefSim:
    """One reference simulation (the harness holds global state: one at a time)."""

    def __init__(self, X, Y, Z, cutoff=3, cage_strain=1.0, K=0.0, efield=(0.0, 0.0, 0.0),
                 constrain_to_x=False, T=300, lengths=(1.0,), prevalence=(1.0,), seed=None):
        self.shape = (X, Y, Z)
        if seed is None:
            seed = (0xDEADBEEF + T) & 0xFFFFFFFF  # src/starrynight-main.c:172
        self.n_neighbours = lib().refh_setup(X, Y, Z, cutoff, cage_strain, K, np.asarray(efield, np.float32),
                                             int(constrain_to_x), int(T), len(lengths),
                                             np.asarray(lengths, np.float32), np.asarray(prevalence, np.float32),
                                             seed & 0xFFFFFFFF)

    def lattice(self) -> np.ndarray:
        X, Y, Z = self.shape
        out = np.zeros((X * Y * Z, 4), np.float32)
        lib().refh_get_lattice(out.reshape(-1))
        return out

    def set_lattice(self, lat4: np.ndarray) -> None:
        lib().refh_set_lattice(np.ascontiguousarray(lat4, np.float32).reshape(-1))

    def mc_moves(self, n: int) -> None:
        lib().refh_mc_moves(int(n))

    def counts(self):
        a, r = ctypes.c_ulonglong(0), ctypes.c_ulonglong(0)
        lib().refh_counts(ctypes.byref(a), ctypes.byref(r))
        return a.value, r.value

    def beta(self) -> float:
        return lib().refh_beta()

    def site_energy(self, x, y, z, new3) -> float:
        return lib().refh_site_energy(x, y, z, np.asarray(list(new3) + [0.0], np.float32))

    def neighbours(self):
        mx = 20000
        dxyz = np.zeros(3 * mx, np.int32)
        d = np.zeros(mx, np.float32)
        n = lib().refh_neighbours(dxyz, d, mx)
        return dxyz[: 3 * n].reshape(n, 3), d[:n]

    def observables(self):
        a, b = ctypes.c_double(0.0), ctypes.c_double(0.0)
        lib().refh_observables(ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def init_pattern(self, name: str) -> None:
        """The reference's InitialLattice pattern (src/starrynight-lattice.c:39-137); lengths untouched."""
        if lib().refh_init_pattern(name.encode()) != 0:
            raise ValueError("unknown pattern %r" % name)

    def potential_map(self) -> np.ndarray:
        out = np.zeros(int(np.prod(self.shape)), np.float64)
        lib().refh_potential_map(out)
        return out

    def efield_map(self, cutoff: int, half: bool = False) -> np.ndarray:
        out = np.zeros(int(np.prod(self.shape)), np.float64)
        lib().refh_efield_map(int(cutoff), int(bool(half)), out)
        return out

    def write(self, kind: str, path: str) -> None:
        """One of the reference's writers (src/starrynight-analysis.c) on the current lattice."""
        if lib().refh_write(kind.encode(), path.encode()) != 0:
            raise ValueError("writer %r failed" % kind)

    def capture(self, kind: str, path: str) -> None:
        """stderr of outputlattice_dumb_terminal / recombination_calculator(stderr) into path."""
        if lib().refh_capture(kind.encode(), path.encode()) != 0:
            raise ValueError("capture %r failed" % kind)
