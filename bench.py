"""Benchmark of the Metropolis dipole-lattice sweep on one GB300.

Headline workload (one "step" = one Metropolis sweep of the lattice):
  256x256x256 lattice of float3 unit dipoles, solid solution with occupancy
  Bernoulli(0.7) from the seed (vacancies are zero dipoles), cutoff r_c = 3
  (122 neighbours), CageStrain 1, Efield (0, 0, 0.1), T = 150 K, with a full
  energy recompute every 50 sweeps (FP32 local fields, FP64 sums) checking the
  running FP64 total for drift.  Synthetic: generated on the device from the
  seed; the reference has no dataset.

Metric: attempted Metropolis updates of occupied sites per second
("dipole site-updates/s"), whole job.  `value` is device-resident (lattice in
HBM, CUDA events on the library's stream around K sweeps, the periodic
recompute included pro rata); `e2e` goes through the C ABI with pinned HOST
buffers every step: upload the lattice, one sweep that writes each block's
final sites into the host buffer as the block ends (sn_gpu_sweep_download),
read the observables -- the drop-in for one MC_moves(X*Y*Z) call of the
reference on a host lattice.

`configs` holds one sub-record per workload of the benchmark table (small
cubic lattice; the headline; the 64-replica table; the 128^3 cutoff-4
differentiable case; the 16 x 96^3 cutoff-5 hysteresis table with a 2048^2
slab), each with its own rate, roofline fraction and the CPU rate of the
reference algorithm on the same parameters.

`--impl reference` times the reference's CPU algorithm (random-sequential
MC_move with MT19937, src/starrynight-montecarlo-core.c:143-191) on the host
cores through the CPU oracle, one process per core as the reference's own
GNU-parallel runs do, on the same lattice and parameters.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "workload": "256^3 solid solution p=0.7, r_c=3, Efield=(0,0,0.1), T=150K, recompute every 50 sweeps",
    "X": 256, "Y": 256, "Z": 256, "cutoff": 3, "occupancy": 0.7, "efield": [0.0, 0.0, 0.1], "T": 150.0,
    "cage_strain": 1.0, "dipole": 1.0, "seed": 20241203, "recompute_every": 50,
    "l2": "inputs larger than L2 (lattice 268 MB > 129 MB L2)",
}
BATCHED = {"replicas": 64, "sizes": [32, 48, 64, 96, 128], "T_range": [50.0, 500.0], "Ez_range": [0.0, 0.2],
           "cutoff": 3, "seed": 777}
METRIC = "dipole site-updates/s on 1 GB300 (batched vs plain), energy err vs FP64"

# CPU samples of the reference algorithm for each sub-record: one lattice per
# host process with these parameters (the batched table's sizes are close in
# rate per move; its middle temperature stands for the ladder).
CPU_CASES = {
    "plain32": dict(X=32, Y=32, Z=32, cutoff=3, T=300, efield=(0.0, 0.0, 0.0), cage_strain=1.0, occupancy=1.0,
                    moves=400_000),
    "batched64": dict(X=64, Y=64, Z=64, cutoff=3, T=158, efield=(0.0, 0.0, 0.1), cage_strain=1.0, occupancy=1.0,
                      moves=400_000),
    "diff128": dict(X=128, Y=128, Z=128, cutoff=4, T=300, efield=(0.05, 0.0, 0.05), cage_strain=0.5,
                    occupancy=0.9, moves=200_000),
    "hysteresis96": dict(X=96, Y=96, Z=96, cutoff=5, T=300, efield=(0.0, 0.0, 0.3), cage_strain=1.0,
                         occupancy=1.0, moves=100_000),
}


def flops_per_update(n_nb: int) -> int:
    """Algorithmic FP32 work of one site-update: 9 FMA per neighbour through the
    symmetric offset tensor plus 64 for cage strain, field, dE, proposal and accept."""
    return 18 * n_nb + 64


# ---------------------------------------------------------------------------
# distributed plumbing (N > 1: independent replicas per rank, weak scaling)
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)


def dist_barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(ws, v: float, op) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op))
    return float(t.item())


def dist_max(ws, v: float) -> float:
    return _reduce(ws, v, "MAX")


def dist_sum(ws, v: float) -> float:
    return _reduce(ws, v, "SUM")


# ---------------------------------------------------------------------------
# clocks during the timed region: NVML read every 10 ms by a thread (the GPU is
# found by its UUID, so CUDA_VISIBLE_DEVICES cannot make it read another GPU);
# nvidia-smi at 20 ms where NVML cannot be loaded.  Reading only: no setting
# of the GPU is changed.
class _NvmlSampler:
    NAMES = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, uuid: str, period_s: float = 0.01):
        self.nvml = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nvml.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.dev = ctypes.c_void_p()
        if self.nvml.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.dev)) != 0:
            raise OSError("GPU %s not found by NVML" % uuid)
        self.period = period_s
        self.samples = []
        self.stop = threading.Event()
        self.thread = threading.Thread(target=self._run, daemon=True)
        mx = ctypes.c_uint(0)
        self.nvml.nvmlDeviceGetMaxClockInfo(self.dev, 1, ctypes.byref(mx))  # NVML_CLOCK_SM
        self.max_mhz = mx.value
        fn = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons

    def _run(self):
        clk, rs = ctypes.c_uint(0), ctypes.c_ulonglong(0)
        while not self.stop.is_set():
            if self.nvml.nvmlDeviceGetClockInfo(self.dev, 1, ctypes.byref(clk)) == 0:
                self.reasons_fn(self.dev, ctypes.byref(rs))
                self.samples.append((float(clk.value), int(rs.value)))
            time.sleep(self.period)

    def start(self):
        self.thread.start()

    def finish(self) -> dict:
        self.stop.set()
        self.thread.join(timeout=2)
        self.nvml.nvmlShutdown()
        reasons = sorted({n for _, r in self.samples for bit, n in self.NAMES.items() if r & bit})
        sm = [c for c, _ in self.samples]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(self.max_mhz),
                "reasons": reasons, "samples": len(sm), "period_ms": 1e3 * self.period, "source": "nvml"}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.nv = None
        self.path = os.path.join("/tmp", "sn_clocks_%d_%d.csv" % (os.getpid(), device))

    def __enter__(self):
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(self.device).uuid)
            self.nv = _NvmlSampler(uuid if uuid.startswith("GPU-") else "GPU-" + uuid)
            self.nv.start()
            return self
        except Exception:
            self.nv = None
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nv is not None:
            self.result = self.nv.finish()
            return
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.nv is not None:
            return self.result
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "period_ms": 20, "source": "nvidia-smi"}


# ---------------------------------------------------------------------------
def read_traffic():
    """DRAM bytes per launch of the headline sweep kernel from the machine-readable
    ncu capture record (profiles/sweep_flow_256cubed.json), with the commit and
    kernel it was captured on."""
    path = os.path.join(ROOT, "profiles", "sweep_flow_256cubed.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch"), {k: d.get(k) for k in ("kernel", "commit", "command")}
    except (OSError, ValueError):
        return None, None


def make_sim(sn, rank=0):
    w = WORKLOAD
    params = sn.ModelParams(cutoff=w["cutoff"], cage_strain=w["cage_strain"], efield=w["efield"],
                            dipoles=(w["dipole"], 0.0), prevalence=(w["occupancy"], 1.0 - w["occupancy"]),
                            seed=w["seed"] + 1000 * rank)
    sim = sn.Simulation(params, [sn.Replica(w["X"], w["Y"], w["Z"], T=w["T"], seed=w["seed"] + 1000 * rank)])
    sim.init_lattice(0)
    return sim


def batched_replicas(sn):
    b = BATCHED
    rng = np.random.default_rng(b["seed"])
    sizes = rng.choice(b["sizes"], size=b["replicas"])
    T = np.geomspace(b["T_range"][0], b["T_range"][1], b["replicas"])
    Ez = rng.uniform(b["Ez_range"][0], b["Ez_range"][1], size=b["replicas"])
    return [sn.Replica(int(L), int(L), int(L), T=float(t), efield=(0.0, 0.0, float(e)), seed=b["seed"] + i)
            for i, (L, t, e) in enumerate(zip(sizes, T, Ez))]


def occupied(sim, nrep):
    return [int((sim.download(r)[1] > 0).sum()) for r in range(nrep)]


def table_flops(sn, sim, reps, cutoff):
    """Algorithmic flops of one sweep of a replica table: sum of occupied sites x F(r_c, 2D or 3D)."""
    occ = occupied(sim, len(reps))
    F = [flops_per_update(sn.neighbour_count(cutoff, r.Z)) for r in reps]
    return sum(occ), float(sum(o * f for o, f in zip(occ, F)))


def run_batched(sn, peak, steps=20):
    """Batched replica table (64 uneven lattices swept by the same launches)
    vs the same lattices swept one handle at a time."""
    reps = batched_replicas(sn)
    params = sn.ModelParams(cutoff=BATCHED["cutoff"], cage_strain=1.0, seed=BATCHED["seed"])
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        occ, flops = table_flops(sn, sim, reps, BATCHED["cutoff"])
        sim.set_exchange(10)
        sim.sweep(3)
        ms = sim.sweep_timed(steps)
    batched = occ * steps / (ms * 1e-3)
    tot_ms = 0.0
    for r in reps:
        with sn.Simulation(params, [r]) as one:
            one.init_lattice(0)
            one.sweep(2)
            tot_ms += one.sweep_timed(steps)
    plain = occ * steps / (tot_ms * 1e-3)
    return {"workload": "64 lattices from {32,48,64,96,128}^3, T log-spaced 50-500 K, Ez~U[0,0.2], r_c=3, exchange "
                        "every 10 sweeps, one dataflow launch per sweep under a captured CUDA graph",
            "replicas": len(reps), "sites": occ, "value": batched, "unit": "site-updates/s", "steps": steps,
            "ms_per_step": ms / steps, "plain_value": plain, "batched_over_plain": batched / plain,
            "roofline_frac": flops * steps / (ms * 1e-3) / 1e12 / peak,
            "note": "plain = the same lattices swept one handle at a time"}


def run_plain32(sn, peak, steps=200):
    params = sn.ModelParams(cutoff=3, cage_strain=1.0, seed=11)
    rep = sn.Replica(32, 32, 32, T=300.0, seed=11)
    with sn.Simulation(params, [rep]) as sim:
        sim.init_lattice(0)
        occ, flops = table_flops(sn, sim, [rep], 3)
        sim.sweep(5)
        ms = sim.sweep_timed(steps)
    return {"workload": "32^3 all occupied, r_c=3, CageStrain 1, Efield 0, T=300 K", "value": occ * steps / (ms * 1e-3),
            "unit": "site-updates/s", "steps": steps, "ms_per_step": ms / steps,
            "roofline_frac": flops * steps / (ms * 1e-3) / 1e12 / peak,
            "note": "32768 sites fill a fraction of the GPU; the 64-replica table is the batched form of this case"}


def run_diff128(sn, peak, steps=20):
    params = sn.ModelParams(cutoff=4, cage_strain=0.5, efield=(0.05, 0.0, 0.05), dipoles=(1.0, 0.0),
                            prevalence=(0.9, 0.1), seed=128)
    rep = sn.Replica(128, 128, 128, T=300.0, seed=128)
    with sn.Simulation(params, [rep]) as sim:
        sim.init_lattice(0)
        occ, flops = table_flops(sn, sim, [rep], 4)
        sim.sweep(5)
        ms = sim.sweep_timed(steps)
        sim.adjoint(0, grad=False)
        t0 = time.perf_counter()
        for _ in range(5):
            sim.adjoint(0, grad=False)
        adj_ms = (time.perf_counter() - t0) * 1e3 / 5
        sim.quench(0, 2, 0.05)
        t0 = time.perf_counter()
        sim.quench(0, 20, 0.05)
        q_ms = (time.perf_counter() - t0) * 1e3 / 20
    return {"workload": "128^3 p=0.9, r_c=4, CageStrain 0.5, Efield (0.05,0,0.05), T=300 K sweeps; adjoint dE/dp and "
                        "dE/d(params); T=0 quench steps", "value": occ * steps / (ms * 1e-3), "unit": "site-updates/s",
            "steps": steps, "ms_per_step": ms / steps, "roofline_frac": flops * steps / (ms * 1e-3) / 1e12 / peak,
            "adjoint_ms": adj_ms, "quench_step_ms": q_ms,
            "note": "adjoint and quench times are host wall time per call (each call ends with its FP64 sums on the "
                    "host)"}


def run_hysteresis96(sn, peak, field_steps=2, sweeps_per_step=20):
    reps = [sn.Replica(96, 96, 96, T=300.0, seed=960 + i) for i in range(16)]
    reps.append(sn.Replica(2048, 2048, 1, T=300.0, seed=2048))
    params = sn.ModelParams(cutoff=5, cage_strain=1.0, seed=96)
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        occ, flops = table_flops(sn, sim, reps, 5)
        sim.sweep(3)
        ms = 0.0
        ramp = [0.3 * (1.0 - abs(1.0 - 4.0 * (k + 1) / 400.0)) for k in range(field_steps)]  # triangle wave start
        for ez in ramp:
            for i in range(len(reps)):
                sim.set_field(i, (0.0, 0.0, ez))
            ms += sim.sweep_timed(sweeps_per_step)
            sim.observables()
    n = field_steps * sweeps_per_step
    return {"workload": "16 x 96^3 r_c=5 + one 2048^2 slab in one handle, T=300 K, Efield_z triangle ramp, "
                        "20 sweeps per field step", "value": occ * n / (ms * 1e-3), "unit": "site-updates/s",
            "steps": n, "ms_per_step": ms / n, "roofline_frac": flops * n / (ms * 1e-3) / 1e12 / peak,
            "note": "F(5) = 9316 flop per 3D update, 1504 per slab update (80 in-plane neighbours)"}


# ---------------------------------------------------------------------------
# CPU: the reference algorithm through the oracle port.  One worker process
# per host core holds its own lattice (initialised once); a step is a
# bounded batch of MC_move calls in every worker.
_CPU = {}


def _cpu_init(seed_base, case):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    c = case
    m = O.make_model(c["X"], c["Y"], c["Z"], c["cutoff"], T=int(c["T"]), efield=tuple(c["efield"]),
                     cage_strain=c["cage_strain"])
    mt = O.MTState((seed_base + os.getpid()) & 0xFFFFFFFF)
    p = c["occupancy"]
    lat = O.ref_init_random(m, mt, (1.0, 0.0), (p, 1.0 - p))
    lat[lat[:, 3] == 0, :3] = 0.0  # vacancies are zero dipoles
    O.ref_mc_moves(m, lat, mt, 1000)
    _CPU.update(O=O, m=m, mt=mt, lat=lat)


def _cpu_step(moves):
    c = _CPU
    a, r = c["O"].ref_mc_moves(c["m"], c["lat"], c["mt"], moves)
    return a + r  # attempted moves on occupied sites


def headline_case():
    w = WORKLOAD
    return dict(X=w["X"], Y=w["Y"], Z=w["Z"], cutoff=w["cutoff"], T=w["T"], efield=tuple(w["efield"]),
                cage_strain=w["cage_strain"], occupancy=w["occupancy"])


class CpuPool:
    def __init__(self, procs, case=None):
        self.procs = procs
        case = case or headline_case()
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(procs, initializer=_cpu_init, initargs=(0xDEADBEEF + int(case["T"]), case))
        self.pool.map(_cpu_step, [1] * procs)  # wait until every worker is initialised

    def step(self, moves):
        t0 = time.perf_counter()
        upd = sum(self.pool.map(_cpu_step, [moves] * self.procs, chunksize=1))
        return upd, time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_rate(case, moves):
    procs = host_cores()
    pool = CpuPool(procs, case)
    upd, dt = pool.step(moves)
    pool.close()
    return {"value": upd / dt, "unit": "site-updates/s", "cores": procs, "kind": "port",
            "sample": "%d random-sequential MC_move calls in each of %d processes (one per host core), each on its own "
                      "%dx%dx%d lattice, r_c=%d, T=%g K" % (moves, procs, case["X"], case["Y"], case["Z"],
                                                            case["cutoff"], case["T"])}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    procs = host_cores()
    moves = args.ref_moves
    pool = CpuPool(procs)
    for _ in range(args.warmup):
        pool.step(moves)
    tot_upd, tot_t = 0, 0.0
    for _ in range(args.steps):
        upd, dt = pool.step(moves)
        tot_upd += upd
        tot_t += dt
    pool.close()
    value = tot_upd / tot_t
    line = {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "site-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
        "data": "synthetic", "config": {k: WORKLOAD[k] for k in WORKLOAD},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": procs, "kind": "port",
                         "sample": "per step %d random-sequential MC_move calls in each of %d processes (one per "
                                   "host core), each on its own 256^3 lattice" % (moves, procs)},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def site_energy_accuracy(site32, site64, occm):
    """FP32-field site energies against the all-FP64 pass on every occupied site."""
    a, b = site32[occm], site64[occm]
    err = np.abs(a - b)
    mag = np.abs(b)
    small = mag < 1.0
    rel_unfloored = err[~small] / mag[~small] if (~small).any() else np.zeros(1)
    return {"site_energy_rel_err_max": float((err / np.maximum(mag, 1.0)).max()),
            "site_energy_rel_err_mean": float((err / np.maximum(mag, 1.0)).mean()),
            "site_energy_abs_err_max": float(err.max()),
            "site_energy_rel_floor": 1.0,
            "site_energy_rel_err_max_unfloored_abs_e_ge_1": float(rel_unfloored.max()),
            "sites_abs_e_lt_1_fraction": float(small.mean()),
            "sites_abs_e_lt_1_abs_err_max": float(err[small].max()) if small.any() else 0.0,
            "sites_abs_e_lt_1_rel_err_max_unfloored": float((err[small] / np.maximum(mag[small], 1e-30)).max())
            if small.any() else 0.0,
            "site_energy_note": "FP32-field site energies vs the all-FP64 pass on every occupied site; relative error "
                                "with |e| floored at 1 energy unit (k_B*300K), and unfloored on both sides of |e| = 1"}


def run_ours(args, ws, rank, local):
    import torch
    import starrynight_gb300 as sn
    torch.cuda.set_device(local)
    sn.build()
    dist_init(ws, "nccl")
    w = WORKLOAD
    sim = make_sim(sn, rank)
    every = w["recompute_every"]
    sim.set_recompute(every, "fp32")
    N = w["X"] * w["Y"] * w["Z"]
    xyz, ln = sim.download(0)
    occ = int((ln > 0).sum())
    del xyz
    sim.sweep(args.warmup)
    # one periodic recompute timed alone, to charge the timed window its share
    torch.cuda.synchronize()
    rst = torch.cuda.ExternalStream(sim.stream_ptr())
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(rst)
    sim.recompute("fp32")
    r1.record(rst)
    r1.synchronize()
    rec_ms = r0.elapsed_time(r1)
    s0 = sim.sweep_count()
    l0 = sim.launches()
    dist_barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        win_ms = sim.sweep_timed(args.steps)
    dist_barrier(ws)
    l1 = sim.launches()
    s1 = sim.sweep_count()
    in_window = s1 // every - s0 // every
    ms = win_ms - in_window * rec_ms + (args.steps / every) * rec_ms
    ms = dist_max(ws, ms)
    total_upd = dist_sum(ws, float(occ) * args.steps)
    value = total_upd / (ms * 1e-3)
    drift, nchk = sim.drift()
    acc_n, rej_n = sim.sweep(5, counts=True)  # acceptance ratio, outside the timed region
    # accuracy: running total vs a full FP64 recompute, FP32-field site energies vs FP64
    obs = sim.observables()
    E_run = obs["E_per_site"][0] * N
    E64, site64 = sim.energy(0, "fp64", site=True)
    E32, site32 = sim.energy(0, "fp32", site=True)
    acc_info = {"acceptance_ratio": acc_n / max(1, acc_n + rej_n),
                "running_vs_fp64_rel": abs(E_run - E64) / abs(E64), "max_drift_fp32_checks": drift}
    acc_info.update(site_energy_accuracy(site32, site64, ln > 0))
    del site32, site64
    # dominant kernel: one launch of the sweep kernel, timed alone
    # The kernels of one sweep, timed alone: the sweep kernel (launch_ms) and,
    # for the cached-field sweep, the proposal kernel before it.  The roofline
    # takes the whole sweep (every kernel of it, events around the sweep), so
    # moving work into a separate kernel cannot raise it.
    launch_ms, sweep_ms, nl = sim.phase_times(5)
    sched = sim.schedule(0)
    nnb = sn.neighbour_count(w["cutoff"], w["Z"])
    F = flops_per_update(nnb)
    peak, clk_nom = sn.fp32_peak()
    achieved = occ * F / (sweep_ms * 1e-3) / 1e12
    traffic, traffic_src = read_traffic()
    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hx = torch.empty(3 * N, dtype=torch.float32, pin_memory=True)
        hl = torch.empty(N, dtype=torch.float32, pin_memory=True)
        sim.download_ptr(0, hx.data_ptr(), hl.data_ptr())
        for _ in range(3):
            sim.upload_ptr(0, hx.data_ptr(), hl.data_ptr())
            sim.sweep_download(1, [hx.data_ptr()])
            sim.observables()
        dist_barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sim.upload_ptr(0, hx.data_ptr(), hl.data_ptr())
            sim.sweep_download(1, [hx.data_ptr()])
            sim.observables()
        dt = dist_max(ws, time.perf_counter() - t0)
        e2e = {"value": dist_sum(ws, float(occ) * args.e2e_steps) / dt, "unit": "site-updates/s",
               "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 12 * N + 40,
               "step": "upload lattice (xyz+len) from pinned host memory, 1 sweep writing its final xyz into the "
                       "pinned host buffer (sn_gpu_sweep_download), observables"}
    sim.close()
    configs = None
    if not args.no_configs and ws == 1:
        configs = {"plain32": run_plain32(sn, peak), "headline256": None, "batched64": run_batched(sn, peak),
                   "diff128": run_diff128(sn, peak), "hysteresis96": run_hysteresis96(sn, peak)}
        configs["headline256"] = {"workload": w["workload"], "value": value, "unit": "site-updates/s",
                                  "steps": args.steps, "ms_per_step": ms / args.steps,
                                  "roofline_frac": value * F / 1e12 / peak, "note": "the headline line itself"}
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_rate(headline_case(), args.cpu_moves)
        if configs:
            for k, case in CPU_CASES.items():
                configs[k]["cpu_port"] = cpu_rate(case, case["moves"])
            configs["headline256"]["cpu_port"] = cpu
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (site), f64 (accumulation)", "data": "synthetic",
            "config": {k: w[k] for k in w}, "gpu_launches": int(l1 - l0),
            "recompute": {"every": every, "ms": rec_ms, "in_window": int(in_window), "window_ms": win_ms,
                          "charged_ms": ms - (win_ms - in_window * rec_ms),
                          "note": "value charges the timed sweeps steps/every recomputes (the window's own "
                                  "recomputes replaced by that share)"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": "measured FP32 FMA loop in this run (MEASURED_PEAKS.json has no FP32 figure)",
                         "flops_per_update": F, "sweep_ms": sweep_ms, "sweep_kernel_ms": launch_ms,
                         "sweep_method": "cached" if sched["field_cache"] else "stencil",
                         "block": [sched["bx"], sched["by"], sched["bz"]],
                         "note": "achieved = F x occupied sites per sweep / device time of the whole sweep; the "
                                 "cached-field sweep does the stencil work only for accepted moves, so F counts "
                                 "work the stencil form would do"},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "accuracy": acc_info, "configs": configs,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-moves", type=int, default=2_000_000, help="MC_move calls per core for cpu_baseline")
    ap.add_argument("--ref-moves", type=int, default=100_000, help="MC_move calls per core per reference step")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="skip the per-workload sub-records")
    ap.add_argument("--no-batched", action="store_true", help="same as --no-configs (kept for older commands)")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    args.no_configs = args.no_configs or args.no_batched
    ws, rank, local = dist_info()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
