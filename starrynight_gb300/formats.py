"""ctypes binding of ``lib/libsn_io.so`` (``include/sn_io.h``): the reference
program's analysis output formats, written from arrays, and the checkpoint
format.  Host-only C; built by :func:`starrynight_gb300.native.build_io`.

Arrays use the lattice index ``(x*Y+y)*Z+z``; ``xyz`` is ``(N, 3)`` float32.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import os

import numpy as np

from . import native as _native

_LIB = None
_LIBC = None

_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_s = ctypes.c_char_p
_i = ctypes.c_int
_vp = ctypes.c_void_p


class Checkpoint(ctypes.Structure):
    _fields_ = [("X", ctypes.c_int32), ("Y", ctypes.c_int32), ("Z", ctypes.c_int32), ("cutoff", ctypes.c_int32),
                ("sweeps", ctypes.c_uint64), ("seed", ctypes.c_uint64), ("T", ctypes.c_double),
                ("efield", ctypes.c_double * 3), ("accept", ctypes.c_uint64), ("attempt", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["efield"] = tuple(self.efield)
        return d


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = _native.io_path()
        if not os.path.exists(path):
            _native.build_io()
        L = ctypes.CDLL(path)
        grid = [_s, _i, _i, _i]
        for name in ("sn_io_write_dipoles_xyz", "sn_io_write_dipoles_ppm", "sn_io_write_dipoles_svg"):
            getattr(L, name).argtypes = grid + [_f]
        for name in ("sn_io_write_potential_xyz", "sn_io_write_potential_cube", "sn_io_write_potential_pgm",
                     "sn_io_write_field_xyz"):
            getattr(L, name).argtypes = grid + [_d]
        L.sn_io_append_rdf.argtypes = [_s, _i, _d, _d, _i64, _i]
        L.sn_io_recombination.argtypes = [_vp, _vp, _i, _i, _i, _d, _i]
        L.sn_io_dumb_terminal.argtypes = [_vp, _i, _i, _i, _f, _vp, _d, _i, ctypes.POINTER(ctypes.c_float)]
        L.sn_io_write_checkpoint.argtypes = [_s, ctypes.POINTER(Checkpoint), _f, _f]
        L.sn_io_read_checkpoint.argtypes = [_s, ctypes.POINTER(Checkpoint), _vp, _vp]
        _LIB = L
    return _LIB


def _libc():
    global _LIBC
    if _LIBC is None:
        _LIBC = ctypes.CDLL(ctypes.util.find_library("c"))
        _LIBC.fopen.restype = _vp
        _LIBC.fopen.argtypes = [_s, _s]
        _LIBC.fclose.argtypes = [_vp]
    return _LIBC


def _ck(rc: int, path) -> None:
    if rc != 0:
        raise OSError("libsn_io: cannot write %s (%d)" % (path, rc))


def _grid(path, shape):
    X, Y, Z = (int(v) for v in shape)
    return os.fsencode(path), X, Y, Z


def _xyz(xyz):
    return np.ascontiguousarray(xyz, np.float32).reshape(-1)


def _map(a):
    return np.ascontiguousarray(a, np.float64).reshape(-1)


def write_dipoles_xyz(path, shape, xyz):
    _ck(lib().sn_io_write_dipoles_xyz(*_grid(path, shape), _xyz(xyz)), path)


def write_dipoles_ppm(path, shape, xyz):
    _ck(lib().sn_io_write_dipoles_ppm(*_grid(path, shape), _xyz(xyz)), path)


def write_dipoles_svg(path, shape, xyz):
    _ck(lib().sn_io_write_dipoles_svg(*_grid(path, shape), _xyz(xyz)), path)


def write_potential_xyz(path, shape, pot):
    _ck(lib().sn_io_write_potential_xyz(*_grid(path, shape), _map(pot)), path)


def write_potential_cube(path, shape, pot):
    _ck(lib().sn_io_write_potential_cube(*_grid(path, shape), _map(pot)), path)


def write_potential_pgm(path, shape, pot):
    _ck(lib().sn_io_write_potential_pgm(*_grid(path, shape), _map(pot)), path)


def write_field_xyz(path, shape, magnitude):
    _ck(lib().sn_io_write_field_xyz(*_grid(path, shape), _map(magnitude)), path)


def append_rdf(path, cutoff, fe_sum, afe_sum, count, T):
    _ck(lib().sn_io_append_rdf(os.fsencode(path), int(cutoff), _map(fe_sum), _map(afe_sum),
                               np.ascontiguousarray(count, np.int64), int(T)), path)


def _with_file(path, fn):
    c = _libc()
    fp = c.fopen(os.fsencode(path), b"w")
    if not fp:
        raise OSError("cannot open %s" % path)
    try:
        return fn(fp)
    finally:
        c.fclose(fp)


def recombination(path, shape, pot, T, art: bool = True):
    """recombination_calculator's log lines (and, with art, its pictures) into path."""
    X, Y, Z = (int(v) for v in shape)
    _ck(_with_file(path, lambda fp: lib().sn_io_recombination(fp, fp if art else None, X, Y, Z, _map(pot), int(T))),
        path)


def dumb_terminal(path, shape, xyz, length, pot, T) -> float:
    X, Y, Z = (int(v) for v in shape)
    dmax = ctypes.c_float(0.0)
    ln = None if length is None else np.ascontiguousarray(length, np.float32).reshape(-1)
    _ck(_with_file(path, lambda fp: lib().sn_io_dumb_terminal(
        fp, X, Y, Z, _xyz(xyz), ln.ctypes.data if ln is not None else None, _map(pot), int(T), ctypes.byref(dmax))),
        path)
    return dmax.value


def write_checkpoint(path, header: dict, xyz, length) -> None:
    h = Checkpoint()
    for k, v in header.items():
        if k == "efield":
            for i in range(3):
                h.efield[i] = float(v[i])
        else:
            setattr(h, k, v)
    _ck(lib().sn_io_write_checkpoint(os.fsencode(path), ctypes.byref(h), _xyz(xyz),
                                     np.ascontiguousarray(length, np.float32).reshape(-1)), path)


def read_checkpoint(path, shape=None):
    """(header dict, xyz (N,3), length (N,)); shape (X,Y,Z) is checked when given."""
    h = Checkpoint()
    rc = lib().sn_io_read_checkpoint(os.fsencode(path), ctypes.byref(h), None, None)
    if rc != 0:
        raise ValueError("not a checkpoint: %s (%d)" % (path, rc))
    if shape is not None:
        h.X, h.Y, h.Z = (int(v) for v in shape)
    N = int(h.X) * int(h.Y) * int(h.Z)
    xyz = np.zeros((N, 3), np.float32)
    ln = np.zeros(N, np.float32)
    rc = lib().sn_io_read_checkpoint(os.fsencode(path), ctypes.byref(h), xyz.ctypes.data, ln.ctypes.data)
    if rc == -3:
        raise ValueError("checkpoint %s holds a different lattice size" % path)
    if rc != 0:
        raise ValueError("corrupt checkpoint: %s (%d)" % (path, rc))
    return h.as_dict(), xyz, ln
