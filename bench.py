#!/usr/bin/env python3
"""Benchmark of the GB300 MD step (aggregate atom-steps/s, batched vs plain).

Default workload: the batched ensemble — 256 independent seeded poly-alanine
systems, chain lengths log-uniform in 50–800 residues (500–8,000 atoms), each
with its own Philox stream, advanced together (one launch per phase, CUDA
graph).  One "step" is one MD step of every resident system.

Printed (rank 0, one JSON line): value = whole-job device throughput with the
state resident in HBM (CUDA events on the library's stream around a graph of K
steps); e2e = the same metric through the C ABI with host state uploaded from
pinned memory and read back every step; roofline of the force kernel (CUDA
events around every force launch inside the timed graph); the plain
one-system-at-a-time loop on a stratified sample of the same systems; the CPU
baseline (the oracle's restatement of the reference step, all host threads).

--impl reference times the reference's CPU step (oracle restatement; the
reference ships no CPU implementation and its Rust host cannot be built) on a
stratified sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "aggregate atom-steps/s, batched vs plain, 1 GB300; p50/p99 job latency"
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12  # SMs x FP32 lanes x FMA x max SM clock


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch256", choices=["batch256", "plain2500", "large100k", "serve", "precision"])
    ap.add_argument("--systems", type=int, default=256)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--equil", type=int, default=400,
                    help="MD steps run on the freshly grown systems before warm-up (equilibration)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg of the default run")
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate, jobs/s")
    ap.add_argument("--serve-hbm-gb", type=float, default=16.0, help="device bytes of the server arena")
    ap.add_argument("--serve-pool", type=int, default=24, help="distinct seeded topologies the jobs draw from")
    ap.add_argument("--drift-systems", type=int, default=16, help="precision study: systems in the drift runs")
    ap.add_argument("--drift-steps", type=int, default=2500, help="precision study: steps of each drift run")
    return ap.parse_args()


# ------------------------------------------------------------------ workload
def workload_sizes(kind: str, nsys: int, seed: int) -> list[tuple[int, int, float]]:
    """(n_chains, n_residues, box_edge) per system."""
    if kind == "plain2500":
        return [(1, 250, 0.0)]
    if kind == "large100k":
        return [(40, 250, 110.0)]
    rng = np.random.default_rng(seed)
    res = np.exp(rng.uniform(math.log(50), math.log(800), size=nsys))
    return [(1, int(round(r)), 0.0) for r in res]


def build_topologies(pq, specs, indices, seed):
    def one(i):
        c, r, box = specs[i]
        return pq.Topology.polyala(c, r, seed=seed + 7919 * i, box_edge=box)

    with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 4)) as ex:
        return list(ex.map(one, indices))


def pair_stats(topo) -> dict:
    """Unique ordinary pairs within 10 Å (P10) and bonded term counts."""
    from scipy.spatial import cKDTree

    p = topo.positions.astype(np.float64)
    t = cKDTree(p)
    within = (int(t.count_neighbors(t, 10.0)) - len(p)) // 2
    excl = len(topo.exclusions) // 2
    return {"atoms": topo.n_atoms, "p10": max(within - excl, 0), "bonds": len(topo.bonds),
            "angles": len(topo.angles), "dihedrals": len(topo.dihedrals), "exceptions": len(topo.exceptions)}


def flops_per_step(st: dict) -> float:
    # algorithmic FLOPs per step of one system: 36 per ordinary pair within the
    # cutoff and per exception, 25/60/90 per bond/angle/torsion term, 60 per atom
    return (36.0 * (st["p10"] + st["exceptions"]) + 25.0 * st["bonds"] + 60.0 * st["angles"] +
            90.0 * st["dihedrals"] + 60.0 * st["atoms"])


def bytes_per_step(st: dict, list_len: float = 0.0) -> float:
    # x (16) + v r/w (32) + int64 forces w/r (48) + per-atom params (16) + x_start (16) per atom
    return st["atoms"] * (128.0 + 4.0 * list_len / 20.0)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        idx = os.environ.get("LOCAL_RANK", "0")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", idx, f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ distributed
def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ------------------------------------------------------------------ CPU legs
def stratified(n: int, k: int) -> list[int]:
    if n <= k:
        return list(range(n))
    return sorted({int(round(i * (n - 1) / (k - 1))) for i in range(k)})


def cpu_reference_rate(pq, topos, steps_cap: int, seconds: float, threads: int) -> tuple[float, str]:
    """Oracle restatement of the reference step loop; returns atom-steps/s."""
    from oracle import oracle as orc

    orc.build()
    p = pq.Params()
    atoms_steps, wall = 0, 0.0
    desc = []
    budget = seconds / max(len(topos), 1)
    for t in topos:
        o = orc.OracleSystem(t.struct(), seed=p.seed, stream=p.stream)
        eng_v = np.zeros((t.n_atoms, 3), np.float32)
        o.set_state(t.positions, eng_v)
        t0 = time.perf_counter()
        o.run(1, threads)
        one = max(time.perf_counter() - t0, 1e-4)
        n = int(max(1, min(steps_cap, budget / one)))
        t0 = time.perf_counter()
        rc = o.run(n, threads)
        dt = time.perf_counter() - t0
        if rc:
            raise RuntimeError(f"oracle step failed ({rc})")
        atoms_steps += t.n_atoms * n
        wall += dt
        desc.append(f"{t.n_atoms}x{n}")
        o.close()
    return atoms_steps / wall, ", ".join(desc)


# ------------------------------------------------------------------ serving
def run_serving(args, pq) -> dict:
    """Poisson stream of MD jobs through the job server (prismq_server_*).

    Jobs: atoms log-uniform in [300, 20000] (chains of 30-2000 residues drawn
    from a pool of seeded topologies at stratified sizes), steps uniform in
    [500, 5000], arrivals Poisson at --serve-rate.  Every job has its own noise
    stream.  Latency = submit -> final state written to the job's host buffers.
    """
    rng = np.random.default_rng(args.seed + 4)
    P = args.serve_pool
    lo, hi = math.log(30), math.log(2000)
    residues = [int(round(math.exp(lo + (i + 0.5) / P * (hi - lo)))) for i in range(P)]
    specs = [(1, r, 0.0) for r in residues]
    pool = build_topologies(pq, specs, list(range(P)), args.seed + 17)
    n = args.serve_jobs
    pick = rng.integers(0, P, size=n)
    steps = rng.integers(500, 5001, size=n)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, size=n))
    srv = pq.Server(int(args.serve_hbm_gb * 2**30), max_systems=1024, chunk_steps=50)
    # warm-up: first admissions tune the force kernel and capture the graph
    for k in range(4):
        srv.submit(pool[k * (P // 4)], 100, pq.Params(stream=900000 + k), want_state=False)
    got = 0
    while got < 4:
        got += len(srv.poll(wait_ms=500))
    base = srv.stats()
    results = []
    t0 = time.perf_counter()
    for k in range(n):
        while True:
            wait = arrivals[k] - (time.perf_counter() - t0)
            if wait <= 0:
                break
            results += srv.poll(wait_ms=max(1, int(wait * 1000)))
        srv.submit(pool[pick[k]], int(steps[k]), pq.Params(stream=k), tag=k)
    t_end = time.time() + 600
    while len(results) < n and time.time() < t_end:
        results += srv.poll(wait_ms=200)
    st = srv.stats()
    srv.close()
    ok = [r for r in results if r.ok]
    lat = np.array([r.latency_s for r in ok])
    wait = np.array([r.start_s - r.submit_s for r in ok])
    first = min(r.submit_s for r in results)
    last = max(r.end_s for r in results)
    atom_steps = float(sum(r.n_atoms * r.steps_done for r in ok))
    atoms = np.array([pool[i].n_atoms for i in pick])
    return {
        "value": atom_steps / (last - first), "unit": "atom-steps/s",
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "mean": float(lat.mean()), "max": float(lat.max())},
        "queue_wait_s": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
        "jobs": n, "completed": len(ok), "failed": len(results) - len(ok),
        "arrival_rate_per_s": args.serve_rate, "span_s": last - first,
        "job_atoms": {"mean": float(atoms.mean()), "min": int(atoms.min()), "max": int(atoms.max())},
        "job_steps_mean": float(steps.mean()),
        "offered_atom_steps_per_s": float((atoms * steps).sum() / arrivals[-1]),
        "gpu_busy_frac": (st["busy_s"] - base["busy_s"]) / max(last - first, 1e-9),
        "chunks": st["chunks"] - base["chunks"], "arena_atoms": st["capacity_atoms"],
        "arena_bytes": st["device_bytes"],
        "sample": f"{n} jobs from a pool of {P} seeded chains (30-2000 residues), Poisson arrivals",
    }


# ------------------------------------------------------------------ precision study
def run_precision(args, pq) -> dict:
    """FP32 production path against the FP64-everywhere run on the batched
    ensemble: per-system force error at identical positions (all systems),
    total-energy drift at gamma = 0 for both precisions and bitwise repeat
    identity (stratified subset), constraint error with SHAKE at 1e-6."""
    specs = workload_sizes("batch256", args.systems, args.seed)
    idx = list(range(len(specs)))
    topos = build_topologies(pq, specs, idx, args.seed)
    atoms = sum(t.n_atoms for t in topos)
    F32, F64 = pq.PRECISION_FP32, pq.PRECISION_FP64
    # ---- force error at identical positions, every system
    b32 = pq.Batch(atoms + 64 * len(topos), len(topos))
    s32 = [b32.add_system(t, pq.Params(stream=i)) for i, t in zip(idx, topos)]
    if args.equil > 0:
        b32.step(args.equil)
    b64 = pq.Batch(atoms + 64 * len(topos), len(topos), precision=F64)
    s64 = [b64.add_system(t, pq.Params(stream=i, precision=F64)) for i, t in zip(idx, topos)]
    states = [b32.get_state(s) for s in s32]
    for s, (x, v) in zip(s64, states):
        b64.set_state(s, x, v)
    from oracle import oracle as orc

    orc.build()

    def rel(a, b):
        return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))

    errs, errs_orc = [], []
    b32.energy(s32[0])  # one evaluation refreshes the forces of every resident system
    b64.energy(s64[0])
    threads = os.cpu_count() or 1
    for k, (a, b) in enumerate(zip(s32, s64)):
        f32, f64 = b32.forces_f64(a), b64.forces_f64(b)
        errs.append(rel(f32, f64))
        # the FP64 oracle with the production pair set (FP32 r^2 inclusion rule)
        t = topos[k]
        x = states[k][0]
        tt = pq.Topology(x, t.masses, t.charges, t.lj_sigma, t.lj_epsilon, t.bonds, t.angles, t.dihedrals,
                         t.exceptions, t.exclusion_offsets, t.exclusions, t.clusters)
        o = orc.OracleSystem(tt.struct())
        fo, _ = o.forces_f64(threads)
        o.close()
        errs_orc.append(rel(f32, fo))
    b32.close()
    b64.close()
    errs, errs_orc = np.array(errs), np.array(errs_orc)
    # ---- gamma = 0 drift and repeat identity on a stratified subset
    pick = stratified(len(topos), args.drift_systems)
    sub = [topos[k] for k in pick]
    sub_atoms = sum(t.n_atoms for t in sub)
    n_steps, n_samp = args.drift_steps, 10

    def drift_run(prec, extra):
        b = pq.Batch(sub_atoms + 64 * len(sub), len(sub), precision=prec)
        sl = [b.add_system(t, pq.Params(stream=k, gamma=0.0, precision=prec, **extra)) for k, t in zip(pick, sub)]
        for s, k in zip(sl, pick):
            x, v = states[k]
            b.set_state(s, x, v)
        e_t = [[] for _ in sl]
        t0 = time.perf_counter()
        for r in range(n_samp + 1):
            if r:
                b.step(n_steps // n_samp)
            for j, s in enumerate(sl):
                e = b.energy(s)  # (re)evaluates every system at unchanged positions
                e_t[j].append(float(e.sum()))
        wall = time.perf_counter() - t0
        fin = [b.get_state_f64(s) for s in sl]
        bond = max(_bond_err(t, fin[j][0]) for j, t in enumerate(sub))
        b.close()
        ts = np.arange(n_samp + 1) * (n_steps // n_samp) * 0.004 / 1000.0  # ns
        slopes = [float(np.polyfit(ts, np.array(e) - e[0], 1)[0]) for e in e_t]
        per_atom = [sl_ / t.n_atoms for sl_, t in zip(slopes, sub)]
        return {"drift_kcal_mol_ns_per_atom": {"median_abs": float(np.median(np.abs(per_atom))),
                                               "max_abs": float(np.max(np.abs(per_atom)))},
                "max_bond_rel_err": bond, "atom_steps_per_s": sub_atoms * n_steps / wall}, fin

    d32, fin32 = drift_run(F32, {})
    _, fin32b = drift_run(F32, {})
    d64, fin64 = drift_run(F64, {"shake_tol": 1e-6, "rattle_tol": 1e-7})
    _, fin64b = drift_run(F64, {"shake_tol": 1e-6, "rattle_tol": 1e-7})
    rep32 = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(fin32, fin32b))
    rep64 = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(fin64, fin64b))
    dev = [float(np.sqrt(((a[0] - b[0]) ** 2).sum(axis=1).mean())) for a, b in zip(fin32, fin64)]
    return {
        "force_rel_rms_fp32_vs_fp64_oracle": {
            "systems": len(errs_orc), "median": float(np.median(errs_orc)),
            "p99": float(np.percentile(errs_orc, 99)), "max": float(errs_orc.max()),
            "note": "same pair set: the oracle admits pairs by the FP32 r^2 rule of the production kernels"},
        "force_rel_rms_fp32_vs_fp64": {
            "systems": len(errs), "median": float(np.median(errs)), "p99": float(np.percentile(errs, 99)),
            "max": float(errs.max()), "over_1e-5": int((errs > 1e-5).sum()),
            "note": "against the FP64-everywhere run, which admits pairs by r^2 in double: pairs whose r^2 "
                    "lies within FP32 rounding of cutoff^2 enter one set only"},
        "drift_gamma0_fp32": d32, "drift_gamma0_fp64_shake1e-6": d64,
        "repeat_bit_identical": {"fp32": bool(rep32), "fp64": bool(rep64)},
        "fp32_vs_fp64_final_rmsd_A": {"median": float(np.median(dev)), "max": float(np.max(dev))},
        "drift_sample": f"{len(sub)} stratified systems ({sub_atoms} atoms), {n_steps} steps "
                        f"({n_steps * 0.004:.0f} ps) at gamma=0 from the equilibrated states, energy every "
                        f"{n_steps // n_samp} steps, slope by least squares",
    }


def _bond_err(topo, x) -> float:
    c = topo.clusters
    err = 0.0
    for k in range(3):
        h = c["hydrogen_atoms"][:, k]
        ok = h >= 0
        if not ok.any():
            continue
        r = np.linalg.norm(x[h[ok]] - x[c["central_atom"][ok]], axis=1)
        L = c["bond_lengths"][ok, k].astype(np.float64)
        err = max(err, float(np.max(np.abs(r - L) / L)))
    return err


# ------------------------------------------------------------------ main legs
def run_reference(args, pq, rank, world):
    if rank != 0:
        return
    specs = workload_sizes(args.workload, args.systems, args.seed)
    idx = stratified(len(specs), 4 if args.workload == "batch256" else 1)
    topos = build_topologies(pq, specs, idx, args.seed)
    threads = os.cpu_count() or 1
    cpu_reference_rate(pq, topos[:1], 2, 1.0, threads)  # warm-up: page in, spin up the thread pool
    value, desc = cpu_reference_rate(pq, topos, max(args.steps, 1), 30.0, threads)
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "impl": "reference", "dtype": "f32",
            "data": "synthetic (seeded poly-alanine systems)",
            "config": {"workload": args.workload, "systems_sampled": len(topos), "sample": desc},
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": f"oracle restatement of the reference step loop on {desc} (atoms x steps)"},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "vs_baseline": None}
    print(json.dumps(line), flush=True)


def run_ours(args, pq, rank, world):
    import torch

    specs = workload_sizes(args.workload, args.systems, args.seed)
    mine = [i for i in range(len(specs)) if i % world == rank]
    topos = build_topologies(pq, specs, mine, args.seed)
    atoms = sum(t.n_atoms for t in topos)
    batch = pq.Batch(max_atoms=atoms + 64 * len(topos), max_systems=len(topos))
    slots = []
    for i, t in zip(mine, topos):
        slots.append(batch.add_system(t, pq.Params(stream=i)))
    if args.equil > 0:
        batch.step(args.equil)  # leave the transient right after growth
    batch.step(max(args.warmup, 3))
    rebuilds0 = sum(batch.counters(s)[1] for s in slots)
    # pair statistics at the warmed-up positions
    stats = []
    for s, t in zip(slots, topos):
        x, _ = batch.get_state(s)
        tt = pq.Topology(x, t.masses, t.charges, t.lj_sigma, t.lj_epsilon, t.bonds, t.angles, t.dihedrals,
                         t.exceptions, t.exclusion_offsets, t.exclusions, t.clusters)
        stats.append(pair_stats(tt))
    flops_launch = sum(flops_per_step(s) for s in stats)
    p10_mean = sum(s["p10"] for s in stats) / max(atoms, 1)
    # ---------------- timed device region
    clocks = ClockSampler()
    launches0 = pq.kernel_launches()
    barrier(world)
    clocks.start()
    total_ms = ctypes.c_float()
    phase_ms = (ctypes.c_float * (5 * args.steps))()
    rc = pq.load().prismq_batch_run_timed(batch.h, args.steps, ctypes.addressof(total_ms),
                                          ctypes.addressof(phase_ms))
    if rc:
        raise pq.PrismQError(rc, pq.load().prismq_last_error().decode())
    clk = clocks.stop()
    barrier(world)
    launches = pq.kernel_launches() - launches0
    # list builds during the timed region (the run advances steps+1 steps)
    builds = sum(batch.counters(s)[1] for s in slots) - rebuilds0
    steps_per_build = len(slots) * (args.steps + 1) / max(builds, 1)
    t_max = max_over_ranks(total_ms.value / 1e3, world)
    total_atoms = sum_over_ranks(float(atoms), world)
    value = total_atoms * args.steps / t_max
    # per step on the main stream: decision + control + OU normals, row
    # builder, rebuilt systems' forces up to the join, integrate; on the second
    # stream the other systems' forces, overlapping the first three
    kernels = ["k_decide+k_control_cells+k_noise", "k_nbr_build", "k_force(rebuilt)+join", "k_integrate",
               "k_force(others, overlapped)"]
    phase_avg = {k: statistics.mean(phase_ms[5 * i + p] for i in range(args.steps)) for p, k in enumerate(kernels)}
    # the roofline's kernel: the force kernel over every system, timed alone
    # right after the timed region (same resident state, same launch shape)
    f_ms = ctypes.c_float()
    rc = pq.load().prismq_batch_time_force(batch.h, 20, ctypes.addressof(f_ms))
    if rc:
        raise pq.PrismQError(rc, pq.load().prismq_last_error().decode())
    f_avg_ms = f_ms.value
    achieved = flops_launch / (f_avg_ms / 1e3) / 1e12
    # ---------------- e2e through the C ABI with pinned host buffers
    span = int(pq.load().prismq_batch_atom_span(batch.h))
    hx = torch.empty(3 * span, dtype=torch.float32, pin_memory=True).numpy()
    hv = torch.empty(3 * span, dtype=torch.float32, pin_memory=True).numpy()
    L = pq.load()
    L.prismq_batch_get_state_all(batch.h, hx.ctypes.data, hv.ctypes.data)
    # each step: upload x, v from the pinned arrays, one step, read x, v back
    # into them -- one C-ABI call (prismq_batch_step_host) with one wait
    for _ in range(2):
        batch.step_host(1, hx, hv, hx, hv)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        rc = L.prismq_batch_step_host(batch.h, 1, hx.ctypes.data, hv.ctypes.data, hx.ctypes.data, hv.ctypes.data)
        if rc:
            raise pq.PrismQError(rc, L.prismq_last_error().decode())
    e2e_t = max_over_ranks(time.perf_counter() - t0, world)
    e2e_value = total_atoms * args.e2e_steps / e2e_t
    # ---------------- plain loop (one system at a time) on a stratified sample
    plain_value = None
    if world == 1 and len(topos) > 1 and not args.no_plain:
        pick = stratified(len(topos), 8)
        a_sum, t_sum = 0, 0.0
        for k in pick:
            eng = pq.NhsAmberFusedEngine(topos[k], pq.Params(stream=mine[k]))
            eng.step(3)
            n = 200
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            eng.step(n)
            dt = time.perf_counter() - t0
            a_sum += topos[k].n_atoms * n
            t_sum += dt
            eng.close()
        plain_value = a_sum / t_sum
    # ---------------- CPU baseline (rank 0, N = 1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pick = stratified(len(topos), 3)
        threads = os.cpu_count() or 1
        rate, desc = cpu_reference_rate(pq, [topos[k] for k in pick], 400, 20.0, threads)
        cpu = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
               "sample": f"oracle restatement of the reference step loop (per-step REF27 rebuild, two FP32 force "
                         f"evaluations per step), systems atoms x steps: {desc}"}
    traffic = None
    tf = ROOT / "profiles" / "force_traffic.txt"
    if tf.exists():
        for ln in tf.read_text().splitlines():
            if ln.startswith("dram_bytes_per_atom_step"):
                traffic = float(ln.split()[1]) * atoms
    roof = {"bound": "fp32", "achieved": achieved, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
            "frac": achieved / FP32_PEAK_TFLOPS, "traffic": traffic,
            "peak_source": "nominal FP32 SIMT peak (152 SMs x 128 lanes x 2 x 2.07 GHz); MEASURED_PEAKS has no FP32 entry",
            "kernel": "k_force", "kernel_avg_ms": f_avg_ms, "flops_per_launch": flops_launch}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        hbm_peak = float(peaks["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        hbm_peak = 6800.0
    step_bytes = sum(bytes_per_step(s) for s in stats)
    hbm = {"achieved_gbs": step_bytes * args.steps / t_max / 1e9, "peak_gbs": hbm_peak,
           "frac": step_bytes * args.steps / t_max / 1e9 / hbm_peak}
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded poly-alanine systems; no dataset)",
        "config": {"workload": args.workload, "systems": len(specs), "atoms_total": int(total_atoms),
                   "atoms_rank0": atoms, "p10_per_atom": p10_mean, "equilibration_steps": args.equil,
                   "steps_per_list_build": steps_per_build, "force_launch_shape": batch.tuning(),
                   "parallelism": f"independent systems sharded over {world} GPU(s)",
                   "l2": "inputs larger than L2 (neighbour rows ~4 KiB/atom, re-read every step)"},
        "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * span,
                "d2h_bytes_per_step": 24 * span, "steps": args.e2e_steps},
        "plain": None if plain_value is None else {"value": plain_value, "unit": "atom-steps/s",
                                                   "batched_over_plain": value / plain_value,
                                                   "sample": "8 stratified systems run alone, 200 steps each"},
        "roofline": roof, "hbm": hbm, "kernel_avg_ms": phase_avg, "gpu_launches": int(launches), "clocks": clk,
        "cpu_baseline": cpu,
    }
    batch.close()
    if rank == 0 and world == 1 and args.workload == "batch256" and not args.no_serve:
        line["serving"] = run_serving(args, pq)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = args_parse()
    import __graft_entry__

    __graft_entry__.build()
    pq = importlib.import_module("prism-q_gb300")
    rank, world, _ = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, pq, rank, world)
    elif args.workload == "precision":
        if rank == 0:
            t0 = time.perf_counter()
            pr = run_precision(args, pq)
            line = {"metric": "precision study: FP32 + int64 fixed-point forces vs FP64 everywhere",
                    "value": pr["force_rel_rms_fp32_vs_fp64_oracle"]["max"],
                    "unit": "relative RMS force error vs the FP64 oracle (max over systems)",
                    "n_gpus": 1, "higher_is_better": False, "dtype": "f32 vs f64",
                    "data": "synthetic (seeded poly-alanine systems; no dataset)",
                    "config": {"workload": "precision", "systems": args.systems, "equilibration_steps": args.equil},
                    "precision": pr, "wall_s": time.perf_counter() - t0}
            print(json.dumps(line), flush=True)
    elif args.workload == "serve":
        if rank == 0:
            launches0 = pq.kernel_launches()
            clocks = ClockSampler()
            clocks.start()
            sv = run_serving(args, pq)
            clk = clocks.stop()
            line = {"metric": METRIC, "value": sv["value"], "unit": "atom-steps/s", "n_gpus": 1,
                    "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded poly-alanine jobs; no dataset)",
                    "config": {"workload": "serve", "jobs": sv["jobs"], "arrival_rate_per_s": sv["arrival_rate_per_s"],
                               "parallelism": "one job server on 1 GPU"},
                    "e2e": {"value": sv["value"], "unit": "atom-steps/s",
                            "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                            "note": "served throughput is end to end: topologies in, final states out"},
                    "serving": sv, "gpu_launches": int(pq.kernel_launches() - launches0), "clocks": clk}
            print(json.dumps(line), flush=True)
    else:
        run_ours(args, pq, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
