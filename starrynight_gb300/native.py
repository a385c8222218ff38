"""Build the CUDA library (``lib/libsn_gpu.so``) and the C host driver.

nvcc compiles every translation unit for sm_103a only, in parallel: the
sweep/field kernels once per cutoff (``-DSN_RC=1..6``), the small kernels,
and the host side of the C ABI.  Outputs stay in-tree under
``starrynight_gb300/lib/``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
MAX_CUTOFF = 6

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
           "-I" + CSRC, "-I" + INCLUDE]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "sn_gpu.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def lib_path() -> str:
    return os.path.join(LIBDIR, "libsn_gpu.so")


def driver_path() -> str:
    return os.path.join(LIBDIR, "starrynight-gpu")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _deps()
    so = lib_path()
    if force or _stale(so, deps):
        jobs = []
        # per cutoff: the sweep kernels, the FP32-field pass and the FP64 pass
        # as three objects, so the large stencils compile in parallel
        for rc in range(MAX_CUTOFF, 0, -1):
            for part in (1, 2, 3):
                obj = os.path.join(LIBDIR, "sn_sweep_rc%d_p%d.o" % (rc, part))
                jobs.append([NVCC] + ARCH + NVFLAGS + ["-DSN_RC=%d" % rc, "-DSN_PART=%d" % part, "-c",
                                                       os.path.join(CSRC, "sn_sweep_inst.cu"), "-o", obj])
        for name in ("sn_kernels", "sn_gpu", "sn_noalloc", "sn_analysis"):
            jobs.append([NVCC] + ARCH + NVFLAGS + ["-c", os.path.join(CSRC, name + ".cu"),
                                                   "-o", os.path.join(LIBDIR, name + ".o")])
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    sys.stderr.write(r.stdout + r.stderr)
        objs = [j[j.index("-o") + 1] for j in jobs]
        tmp = so + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
        os.replace(tmp, so)
    io = build_io(force)
    drv = driver_path()
    dsrc = [os.path.join(PKG, "driver", "starrynight-gpu.c"), os.path.join(PKG, "cfg", "libconfig_min.c")]
    if all(os.path.exists(p) for p in dsrc) and (force or _stale(drv, dsrc + [so, io, os.path.join(INCLUDE, "sn_gpu.h")])):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE, "-I" + os.path.join(PKG, "cfg"), "-o", drv] + dsrc +
             ["-L" + LIBDIR, "-lsn_gpu", "-lsn_io", "-Wl,-rpath,$ORIGIN", "-lm"])
    return so


def io_path() -> str:
    return os.path.join(LIBDIR, "libsn_io.so")


def build_io(force: bool = False) -> str:
    """Host-only output-format and checkpoint library (no CUDA)."""
    os.makedirs(LIBDIR, exist_ok=True)
    io = io_path()
    src = [os.path.join(PKG, "io", "sn_io.c"), os.path.join(INCLUDE, "sn_io.h")]
    if force or _stale(io, src):
        tmp = io + ".tmp"
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-Wall", "-fPIC", "-shared", "-I" + INCLUDE, "-o", tmp,
              src[0], "-lm"])
        os.replace(tmp, io)
    return io


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
