#!/usr/bin/env python3
"""Benchmark of the GB300 MD step (aggregate atom-steps/s, batched vs plain).

Default workload: the batched ensemble — 256 independent seeded poly-alanine
systems, chain lengths log-uniform in 50–800 residues (500–8,000 atoms), each
chain collapsed into a globule at 0.0746 atoms/Å^3 (2,500 atoms in 40 Å) and
given its own Philox stream, advanced together (one launch per phase, CUDA
graph).  One "step" is one MD step of every resident system.  --workload
large100k is the single 100,000-atom system (40 chains packed in a 110 Å
cube), plain2500 one 2,500-atom globule, serve the Poisson job stream,
precision the FP32-vs-FP64 study.

Printed (rank 0, one JSON line): value = whole-job device throughput with the
state resident in HBM (CUDA events on the library's stream around a graph of K
steps); e2e = the same metric through the C ABI with host state uploaded from
pinned memory and read back every step; the roofline of the force kernel (its
average duration launched alone over every system, CUDA events); the plain
one-system-at-a-time loop on a stratified sample of the same systems; the CPU
baseline (the oracle's restatement of the reference step, all host threads)
on a stratified sample at the device arm's equilibrated states.

--gpus N without a launcher starts N ranks through torch.distributed.run;
systems are sharded round-robin over the ranks with no data-path collective.

--impl reference times the reference's CPU step (oracle restatement; the
reference ships no CPU implementation and its Rust host cannot be built) on
the same stratified sample, with inputs from the oracle's own build of the
generator: the product library is not loaded.
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
                    help="MD steps run on the freshly built systems before warm-up (equilibration)")
    ap.add_argument("--cpu-systems", type=int, default=16,
                    help="stratified systems of the workload that the CPU legs time")
    ap.add_argument("--cpu-steps", type=int, default=20, help="steps the device arm's CPU-baseline leg times")
    ap.add_argument("--pair-layout", default="rows", choices=["rows", "tiles"],
                    help="production neighbour-list layout: per-atom rows (default) or cluster-pair tiles")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg of the default run")
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate, jobs/s")
    ap.add_argument("--serve-hbm-gb", type=float, default=16.0, help="device bytes of the server arena")
    ap.add_argument("--serve-pool", type=int, default=64, help="distinct seeded topologies the jobs draw from")
    ap.add_argument("--drift-systems", type=int, default=16, help="precision study: systems in the drift runs")
    ap.add_argument("--drift-steps", type=int, default=2500, help="precision study: steps of each drift run")
    return ap.parse_args()


# ------------------------------------------------------------------ workload
# Atom density of the collapsed chains: 2,500 atoms in a 40 Å globule.
GLOBULE_DENSITY = 2500.0 / (4.0 / 3.0 * math.pi * 20.0 ** 3)


def workload_sizes(kind: str, nsys: int, seed: int) -> list[tuple[int, int, float]]:
    """(n_chains, n_residues, box_edge) per system; box_edge 0 = one globule per chain."""
    if kind == "plain2500":
        return [(1, 250, 0.0)]
    if kind == "large100k":
        return [(40, 250, 110.0)]
    rng = np.random.default_rng(seed)
    res = np.exp(rng.uniform(math.log(50), math.log(800), size=nsys))
    return [(1, int(round(r)), 0.0) for r in res]


def workload_config(args, specs) -> dict:
    """The workload as both arms describe it (inputs only, nothing measured)."""
    geometry = {
        "batch256": "each chain (log-uniform 50-800 residues) collapsed into a globule at %.4f atoms/A^3" % GLOBULE_DENSITY,
        "plain2500": "one 250-residue chain collapsed into a 40 A globule (%.4f atoms/A^3)" % GLOBULE_DENSITY,
        "large100k": "40 chains x 250 residues packed in a 110 A cube (0.0751 atoms/A^3)",
    }.get(args.workload, args.workload)
    return {"workload": args.workload, "systems": len(specs),
            "atoms_total": int(sum(10 * c * r for c, r, _ in specs)), "geometry": geometry,
            "dt_ps": 0.004, "cutoff_A": 10.0, "skin_A": 2.0, "rebuild_interval": 20, "gamma_per_ps": 1.0,
            "temperature_K": 300.0, "hmr": "H 3.024 amu", "equilibration_steps": args.equil,
            "seed": args.seed, "parallelism": f"independent systems sharded over {args.gpus} GPU(s)",
            "l2": "inputs larger than L2 (state + neighbour lists of 10^5-10^6 atoms, re-read every step)"}


def system_seed(seed: int, i: int) -> int:
    return seed + 7919 * i


def build_topologies(gen, specs, indices, seed):
    """gen(n_chains, n_residues, seed, box_edge) -> topology, on a thread pool
    (the generator releases the interpreter while it runs)."""
    def one(i):
        c, r, box = specs[i]
        return gen(c, r, system_seed(seed, i), box)

    with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 4)) as ex:
        return list(ex.map(one, indices))


def library_generator(pq):
    return lambda c, r, seed, box: pq.Topology.polyala_compact(c, r, seed=seed, box_edge=box)


def oracle_generator():
    from oracle import oracle as orc

    return lambda c, r, seed, box: orc.polyala(c, r, seed, box_edge=box, compact=True)


def pair_stats(topo) -> dict:
    """Unique ordinary pairs within 10 Å (P10) and 12 Å (list entries), and bonded term counts."""
    from scipy.spatial import cKDTree

    p = topo.positions.astype(np.float64)
    t = cKDTree(p)
    within = (int(t.count_neighbors(t, 10.0)) - len(p)) // 2
    within12 = (int(t.count_neighbors(t, 12.0)) - len(p)) // 2
    excl = len(topo.exclusions) // 2
    return {"atoms": topo.n_atoms, "p10": max(within - excl, 0), "p12": max(within12 - excl, 0),
            "bonds": len(topo.bonds), "angles": len(topo.angles), "dihedrals": len(topo.dihedrals),
            "exceptions": len(topo.exceptions)}


def flops_per_step(st: dict) -> float:
    # algorithmic FLOPs per step of one system: 36 per ordinary pair within the
    # cutoff and per exception, 25/60/90 per bond/angle/torsion term, 60 per atom
    return (36.0 * (st["p10"] + st["exceptions"]) + 25.0 * st["bonds"] + 60.0 * st["angles"] +
            90.0 * st["dihedrals"] + 60.0 * st["atoms"])


def bytes_per_step(st: dict, steps_per_build: float) -> float:
    # x (16) + v r/w (32) + int64 forces w/r (48) + per-atom params (16) +
    # x_start (16) per atom, plus the list: 4 bytes per entry (both ends of
    # every pair within the 12 Å list radius) written once per build
    return st["atoms"] * 128.0 + 4.0 * 2.0 * st["p12"] / max(steps_per_build, 1.0)


def maxwell_boltzmann(topo, temperature: float, seed: int) -> np.ndarray:
    """Seeded velocities (Å/ps) at `temperature`, centre-of-mass motion removed."""
    kb = 0.0019872041  # kcal/(mol K)
    m = topo.masses.astype(np.float64)
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((topo.n_atoms, 3)) * np.sqrt(418.4 * kb * temperature / m)[:, None]
    v -= (m[:, None] * v).sum(axis=0) / m.sum()
    return v.astype(np.float32)


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
def spawn_ranks(n: int, argv: list[str]) -> int:
    """Run this script as n ranks through torch.distributed.run on 127.0.0.1
    (used when --gpus N > 1 is given without a launcher); returns the exit code."""
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(port), *argv]
    return subprocess.run(cmd).returncode


def dist_setup(n_gpus: int, pq=None):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world != n_gpus:
        raise SystemExit(f"--gpus {n_gpus} but WORLD_SIZE {world}")
    import torch

    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    if pq is not None:
        # the library's CUDA runtime is its own: select its device too, and check it
        pq.set_device(local)
        if pq.device_ordinal() != local:
            raise SystemExit(f"rank {rank}: library device {pq.device_ordinal()} != LOCAL_RANK {local}")
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _reduce(v: float, world: int, op) -> float:
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch.distributed as dist

    return _reduce(v, world, dist.ReduceOp.MAX)


def sum_over_ranks(v: float, world: int) -> float:
    if world == 1:
        return v
    import torch.distributed as dist

    return _reduce(v, world, dist.ReduceOp.SUM)


# ------------------------------------------------------------------ CPU legs
def stratified(n: int, k: int) -> list[int]:
    if n <= k:
        return list(range(n))
    return sorted({int(round(i * (n - 1) / (k - 1))) for i in range(k)})


def cpu_step_rate(systems, steps: int, threads: int) -> tuple[float, float, str]:
    """The oracle's restatement of the reference step loop (per-step REF27
    rebuild, two FP32 force evaluations per step, OpenMP over `threads`).
    One step = one MD step of every system of the sample, in turn.
    systems: [(topology, x, v)].  Returns (atom-steps/s, ms per step, sample)."""
    from oracle import oracle as orc

    orc.build()
    objs = []
    for t, x, v in systems:
        o = orc.OracleSystem(t.struct())
        o.set_state(x, v)
        objs.append(o)
    atoms = sum(t.n_atoms for t, _, _ in systems)
    t0 = time.perf_counter()
    for _ in range(steps):
        for o in objs:
            rc = o.run(1, threads)
            if rc:
                raise RuntimeError(f"oracle step failed ({rc})")
    wall = time.perf_counter() - t0
    for o in objs:
        o.close()
    desc = f"{len(systems)} stratified systems ({atoms} atoms: " + ", ".join(str(t.n_atoms) for t, _, _ in systems) + ")"
    return atoms * steps / wall, wall * 1e3 / steps, desc


# ------------------------------------------------------------------ serving
def run_serving(args, pq) -> dict:
    """Poisson stream of MD jobs through the job server (prismq_server_*).

    Jobs: chains of 30-2,000 residues (300-20,000 atoms, log-uniform), each
    collapsed into a globule, drawn from a pool of --serve-pool seeded
    topologies at stratified sizes; steps uniform in [500, 5000]; arrivals
    Poisson at --serve-rate; every job has its own noise stream and starting
    velocities.  Latency = submit -> final state written to the job's host
    buffers.  The steady-state rate counts the atom-steps done inside the
    middle 60 % of the arrival span, each job's steps spread evenly over its
    residence in the arena.
    """
    rng = np.random.default_rng(args.seed + 4)
    P = args.serve_pool
    lo, hi = math.log(30), math.log(2000)
    residues = [int(round(math.exp(lo + (i + 0.5) / P * (hi - lo)))) for i in range(P)]
    specs = [(1, r, 0.0) for r in residues]
    t_gen = time.perf_counter()
    pool = build_topologies(library_generator(pq), specs, list(range(P)), args.seed + 17)
    t_gen = time.perf_counter() - t_gen
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
    t_end = time.time() + 3600
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
    w0, w1 = first + 0.2 * (arrivals[-1] - arrivals[0]), first + 0.8 * (arrivals[-1] - arrivals[0])
    mid = 0.0
    for r in ok:
        span = max(r.end_s - r.start_s, 1e-9)
        overlap = max(0.0, min(r.end_s, w1) - max(r.start_s, w0))
        mid += r.n_atoms * r.steps_done * overlap / span
    return {
        "value": atom_steps / (last - first), "unit": "atom-steps/s",
        "steady_state_atom_steps_per_s": mid / max(w1 - w0, 1e-9),
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
        "arena_bytes": st["device_bytes"], "pool_build_s": t_gen,
        "sample": f"{n} jobs drawn from a pool of {P} seeded compact chains (30-2000 residues), Poisson arrivals",
    }


# ------------------------------------------------------------------ precision study
def run_precision(args, pq) -> dict:
    """FP32 production path against the FP64-everywhere run on the batched
    ensemble: per-system force error at identical positions (all systems),
    total-energy drift at gamma = 0 for both precisions and bitwise repeat
    identity (stratified subset), constraint error with SHAKE at 1e-6."""
    specs = workload_sizes("batch256", args.systems, args.seed)
    idx = list(range(len(specs)))
    topos = build_topologies(library_generator(pq), specs, idx, args.seed)
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
def cpu_sample(args, specs) -> list[int]:
    """Indices of the stratified systems both CPU legs time."""
    return stratified(len(specs), args.cpu_systems)


def run_reference(args, rank, world):
    """The reference's CPU implementation of the step (the oracle's
    restatement; the reference ships no CPU path and its Rust host cannot be
    built here) on the host cores.  Inputs come from the oracle's own build of
    the generator, so the product library is not loaded; the sampled systems
    start from Maxwell-Boltzmann velocities and are equilibrated for --equil
    steps by the same CPU step before warm-up and timing."""
    if rank != 0:
        return
    specs = workload_sizes(args.workload, args.systems, args.seed)
    idx = cpu_sample(args, specs)
    topos = build_topologies(oracle_generator(), specs, idx, args.seed)
    threads = os.cpu_count() or 1
    from oracle import oracle as orc

    states = []
    for i, t in zip(idx, topos):
        o = orc.OracleSystem(t.struct(), stream=i)
        o.set_state(t.positions, maxwell_boltzmann(t, 300.0, system_seed(args.seed, i)))
        if o.run(args.equil + args.warmup, threads):
            raise RuntimeError("oracle equilibration failed")
        x, v = o.get_state()
        o.close()
        states.append((t, x, v))
    value, ms, desc = cpu_step_rate(states, max(args.steps, 1), threads)
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "impl": "reference",
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded compact poly-alanine systems; no dataset)",
            "config": workload_config(args, specs),
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": f"oracle restatement of the reference step loop (per-step REF27 rebuild, "
                                       f"two FP32 force evaluations per step) on {desc}, each equilibrated "
                                       f"{args.equil} steps; one step = one step of every sampled system"},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def force_traffic(cfg: dict, layout: str) -> tuple[float | None, str | None]:
    """DRAM bytes per force launch from the committed ncu summary of this
    workload, if one exists for it (same workload, atom count and layout)."""
    for f in sorted((ROOT / "profiles").glob("k_force_*.txt")):
        kv = {}
        for ln in f.read_text().splitlines():
            parts = ln.split()
            if len(parts) >= 2 and not ln.startswith("#"):
                kv[parts[0]] = parts[1]
        if kv.get("workload") == cfg["workload"] and kv.get("atoms_total") == str(cfg["atoms_total"]) \
                and kv.get("pair_layout") == layout and "dram_bytes_per_launch" in kv:
            return float(kv["dram_bytes_per_launch"]), str(f.relative_to(ROOT))
    return None, None


def run_ours(args, pq, rank, world):
    import torch

    specs = workload_sizes(args.workload, args.systems, args.seed)
    cfg = workload_config(args, specs)
    mine = [i for i in range(len(specs)) if i % world == rank]
    topos = build_topologies(library_generator(pq), specs, mine, args.seed)
    atoms = sum(t.n_atoms for t in topos)
    batch = pq.Batch(max_atoms=atoms + 64 * len(topos), max_systems=len(topos))
    batch.set_pair_layout(pq.PAIR_TILES if args.pair_layout == "tiles" else pq.PAIR_ROWS)
    slots = []
    for i, t in zip(mine, topos):
        slots.append(batch.add_system(t, pq.Params(stream=i)))
    if args.equil > 0:
        batch.step(args.equil)  # leave the transient right after the compaction
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
    torch.cuda.nvtx.range_push("timed")  # the launches a profiler of the timed region selects
    rc = pq.load().prismq_batch_run_timed(batch.h, args.steps, ctypes.addressof(total_ms),
                                          ctypes.addressof(phase_ms))
    torch.cuda.nvtx.range_pop()
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
    torch.cuda.nvtx.range_push("force_alone")  # the launches a profiler of this kernel selects
    rc = pq.load().prismq_batch_time_force(batch.h, 20, ctypes.addressof(f_ms))
    torch.cuda.nvtx.range_pop()
    if rc:
        raise pq.PrismQError(rc, pq.load().prismq_last_error().decode())
    f_avg_ms = f_ms.value
    achieved = flops_launch / (f_avg_ms / 1e3) / 1e12
    dev = pq.device_info()
    fp32_peak = dev["sms"] * 128 * 2 * dev["sm_clock_khz"] * 1e3 / 1e12
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
            x, v = batch.get_state(slots[k])
            eng.set_positions(x)
            eng.set_velocities(v)
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
    # ---------------- CPU baseline (rank 0, N = 1) on the equilibrated states
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        idx = cpu_sample(args, specs)
        threads = os.cpu_count() or 1
        systems = [(topos[i], *batch.get_state(slots[i])) for i in idx]
        rate, _, desc = cpu_step_rate(systems, args.cpu_steps, threads)
        cpu = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
               "sample": f"oracle restatement of the reference step loop (per-step REF27 rebuild, two FP32 force "
                         f"evaluations per step) on {desc} at the device arm's equilibrated states, "
                         f"{args.cpu_steps} steps"}
    traffic, traffic_src = force_traffic(cfg, args.pair_layout)
    roof = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": achieved / fp32_peak, "traffic": traffic, "traffic_source": traffic_src,
            "peak_source": f"FP32 SIMT peak of the device: {dev['sms']} SMs x 128 lanes x 2 (FMA) x "
                           f"{dev['sm_clock_khz'] / 1e3:.0f} MHz peak SM clock (MEASURED_PEAKS has no FP32 entry)",
            "kernel": "k_force", "kernel_avg_ms": f_avg_ms, "flops_per_launch": flops_launch}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        hbm_peak, hbm_src = float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, ValueError, KeyError):
        hbm_peak, hbm_src = 6800.0, "fallback 6.8 TB/s"
    step_bytes = sum(bytes_per_step(s, steps_per_build) for s in stats)
    hbm = {"achieved_gbs": step_bytes * args.steps / t_max / 1e9, "peak_gbs": hbm_peak, "peak_source": hbm_src,
           "frac": step_bytes * args.steps / t_max / 1e9 / hbm_peak,
           "bytes_per_step": step_bytes}
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded compact poly-alanine systems; no dataset)",
        "config": cfg,
        "measured": {"atoms_rank0": atoms, "p10_per_atom": p10_mean, "steps_per_list_build": steps_per_build,
                     "force_launch_shape": batch.tuning(), "pair_layout": args.pair_layout, "device": dev},
        "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * span,
                "d2h_bytes_per_step": 24 * span, "steps": args.e2e_steps},
        "plain": None if plain_value is None else {"value": plain_value, "unit": "atom-steps/s",
                                                   "batched_over_plain": value / plain_value,
                                                   "sample": "8 stratified systems run alone from their "
                                                             "equilibrated states, 200 steps each"},
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
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # no launcher: start the ranks here, one process per GPU
        sys.exit(spawn_ranks(args.gpus, [str(pathlib.Path(__file__).resolve()), *sys.argv[1:]]))
    if args.impl == "reference":
        # host cores only: the product library is neither built nor loaded
        rank, world, _ = dist_setup(args.gpus)
        run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return
    import __graft_entry__

    __graft_entry__.build()
    pq = importlib.import_module("prism-q_gb300")
    rank, world, _ = dist_setup(args.gpus, pq)
    if args.workload == "precision":
        if rank == 0:
            t0 = time.perf_counter()
            pr = run_precision(args, pq)
            line = {"metric": "precision study: FP32 + int64 fixed-point forces vs FP64 everywhere",
                    "value": pr["force_rel_rms_fp32_vs_fp64_oracle"]["max"],
                    "unit": "relative RMS force error vs the FP64 oracle (max over systems)",
                    "n_gpus": 1, "higher_is_better": False, "dtype": "f32 vs f64",
                    "data": "synthetic (seeded compact poly-alanine systems; no dataset)",
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
                    "vs_baseline": None, "dtype": "f32",
                    "data": "synthetic (seeded compact poly-alanine jobs; no dataset)",
                    "config": {"workload": "serve", "jobs": sv["jobs"], "arrival_rate_per_s": sv["arrival_rate_per_s"],
                               "pool": args.serve_pool, "hbm_gb": args.serve_hbm_gb,
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
