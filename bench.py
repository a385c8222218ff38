"""Benchmark of the Metropolis dipole-lattice sweep on one GB300.

Workload (one "step" = one Metropolis sweep of the lattice):
  256x256x256 lattice of float3 unit dipoles, solid solution with occupancy
  Bernoulli(0.7) from the seed (vacancies are zero dipoles), cutoff r_c = 3
  (122 neighbours), CageStrain 1, Efield (0, 0, 0.1), T = 150 K, with a full
  energy recompute every 50 sweeps (FP32 local fields, FP64 sums) checking the
  running FP64 total for drift.  Synthetic: generated on the device from the
  seed; the reference has no dataset.

Metric: attempted Metropolis updates of occupied sites per second
("dipole site-updates/s"), whole job.  `value` is device-resident (lattice in
HBM, CUDA events on the library's stream around K sweeps); `e2e` goes through
the C ABI with pinned HOST buffers every step: upload the lattice, one sweep
that writes each block's final sites into the host buffer as the block ends
(sn_gpu_sweep_download), read the observables -- the drop-in for one
MC_moves(X*Y*Z) call of the reference on a host lattice.

`--impl reference` times the reference's CPU algorithm (random-sequential
MC_move with MT19937, src/starrynight-montecarlo-core.c:143-191) on the host
cores through the CPU oracle, one process per core as the reference's own
GNU-parallel runs do, on the same lattice and parameters.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
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


def dist_max(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", "sn_clocks_%d_%d.csv" % (os.getpid(), device))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
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
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def read_traffic():
    """DRAM bytes per launch of the sweep kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "sweep_flow_256cubed.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


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


def time_sweeps(sim, torch, n):
    st = torch.cuda.ExternalStream(sim.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    sim.sweep(n)
    e1.record(st)
    e1.synchronize()
    sim.observables()  # raises if a device wait of the timed sweeps gave up (SN_ERR_TIMEOUT)
    return e0.elapsed_time(e1)


def run_batched(sn, torch, steps=20):
    """Batched replica table (64 uneven lattices swept by the same launches)
    vs the same lattices swept one handle at a time."""
    reps = batched_replicas(sn)
    params = sn.ModelParams(cutoff=BATCHED["cutoff"], cage_strain=1.0, seed=BATCHED["seed"])
    occ = sum(r.n_sites for r in reps)
    with sn.Simulation(params, reps) as sim:
        for i in range(len(reps)):
            sim.init_lattice(i)
        sim.set_exchange(10)
        sim.sweep(3)
        ms = time_sweeps(sim, torch, steps)
    batched = occ * steps / (ms * 1e-3)
    tot_ms = 0.0
    for r in reps:
        with sn.Simulation(params, [r]) as one:
            one.init_lattice(0)
            one.sweep(2)
            tot_ms += time_sweeps(one, torch, steps)
    plain = occ * steps / (tot_ms * 1e-3)
    return {"replicas": len(reps), "sites": occ, "value": batched, "plain_value": plain,
            "batched_over_plain": batched / plain, "unit": "site-updates/s",
            "note": "64 lattices from {32,48,64,96,128}^3, T log-spaced 50-500 K, Ez~U[0,0.2], exchange every 10 sweeps;"
                    " plain = the same lattices swept one handle at a time"}


# ---------------------------------------------------------------------------
# CPU: the reference algorithm through the oracle port.  One worker process
# per host core holds its own 256^3 lattice (initialised once); a step is a
# bounded batch of MC_move calls in every worker.
_CPU = {}


def _cpu_init(seed_base):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    w = WORKLOAD
    m = O.make_model(w["X"], w["Y"], w["Z"], w["cutoff"], T=int(w["T"]), efield=w["efield"],
                     cage_strain=w["cage_strain"])
    mt = O.MTState((seed_base + os.getpid()) & 0xFFFFFFFF)
    lat = O.ref_init_random(m, mt, (w["dipole"], 0.0), (w["occupancy"], 1.0 - w["occupancy"]))
    lat[lat[:, 3] == 0, :3] = 0.0  # vacancies are zero dipoles
    O.ref_mc_moves(m, lat, mt, 1000)
    _CPU.update(O=O, m=m, mt=mt, lat=lat)


def _cpu_step(moves):
    c = _CPU
    a, r = c["O"].ref_mc_moves(c["m"], c["lat"], c["mt"], moves)
    return a + r  # attempted moves on occupied sites


class CpuPool:
    def __init__(self, procs):
        self.procs = procs
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(procs, initializer=_cpu_init, initargs=(0xDEADBEEF + int(WORKLOAD["T"]),))
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
def run_ours(args, ws, rank, local):
    import torch
    import starrynight_gb300 as sn
    torch.cuda.set_device(local)
    sn.build()
    dist_init(ws, "nccl")
    w = WORKLOAD
    sim = make_sim(sn, rank)
    sim.set_recompute(w["recompute_every"], "fp32")
    N = w["X"] * w["Y"] * w["Z"]
    xyz, ln = sim.download(0)
    occ = int((ln > 0).sum())
    del xyz
    sim.sweep(args.warmup)
    torch.cuda.synchronize()
    l0 = sim.launches()
    dist_barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_sweeps(sim, torch, args.steps)
    dist_barrier(ws)
    l1 = sim.launches()
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
    occm = ln > 0
    err = np.abs(site32[occm] - site64[occm])
    rel = err / np.maximum(np.abs(site64[occm]), 1.0)
    acc_info = {"acceptance_ratio": acc_n / max(1, acc_n + rej_n),
                "running_vs_fp64_rel": abs(E_run - E64) / abs(E64), "max_drift_fp32_checks": drift,
                "site_energy_rel_err_max": float(rel.max()), "site_energy_rel_err_mean": float(rel.mean()),
                "site_energy_abs_err_max": float(err.max()),
                "site_energy_rel_floor": 1.0,
                "site_energy_note": "FP32-field site energies vs the all-FP64 pass on every occupied site; "
                                    "relative error with |e| floored at 1 energy unit (k_B*300K)"}
    # dominant kernel: one block-colour launch of the sweep kernel, timed alone
    launch_ms, sweep_ms, nl = sim.phase_times(5)
    nnb = sn.neighbour_count(w["cutoff"], w["Z"])
    F = flops_per_update(nnb)
    peak, clk_nom = sn.fp32_peak()
    achieved = (occ / nl) * F / (launch_ms * 1e-3) / 1e12
    traffic = read_traffic()
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
    batched = None
    if not args.no_batched and ws == 1:
        batched = run_batched(sn, torch)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        procs = host_cores()
        pool = CpuPool(procs)
        upd, dt = pool.step(args.cpu_moves)
        pool.close()
        cpu = {"value": upd / dt, "unit": "site-updates/s", "cores": procs, "kind": "port",
               "sample": "%d random-sequential MC_move calls in each of %d processes (one per host core, "
                         "reference algorithm with MT19937), each on its own 256^3 lattice" % (args.cpu_moves, procs)}
    clocks = clk.summary()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "site-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (site), f64 (accumulation)", "data": "synthetic",
            "config": {k: w[k] for k in w}, "gpu_launches": int(l1 - l0),
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "measured FP32 FMA loop in this run (MEASURED_PEAKS.json has no FP32 figure)",
                         "flops_per_update": F, "launch_ms": launch_ms, "launches_per_sweep": nl},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "accuracy": acc_info, "batched": batched,
        }
        print(json.dumps(line), flush=True)
    sim.close()


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
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_info()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
