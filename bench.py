#!/usr/bin/env python
"""Benchmark of the spherical vertex-model Brownian step (vertex-steps/s at N = 100k cells).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the configuration the headline metric is quoted on): FP64 plain overdamped Brownian
dynamics of the spherical vertex model with N = 100,000 cells (199,996 vertices), cell centres
uniform on the sphere of radius sqrt(N / 4 pi) from a seed, initial vertices from their spherical
Voronoi tessellation, A0 = 1, P0 = 3.8, K_A = K_P = 1, T = 0.01, mu = 1, dt = 0.01, T1 threshold
0.04.  A step is one timestep: geometry, forces, Brownian displacement, move onto the sphere and
T1 flips.  The state is prepared with the reference driver's own recipe (sphericalVertex.cpp:104-125):
STAB steps at T = 0 with P0 = 1, then the run parameters; from a raw random-Voronoi start at
N >= 20k the reference model itself develops inverted cells and diverges, while the stabilised
start relaxes normally.  Timing starts after the stabilisation and an untimed equilibration.

ours: `value` is device-resident throughput over K steps, each timed with CUDA events on the
model's stream after an L2 flush (the model state, ~40 MB, would otherwise stay in the 129 MB L2);
`e2e` is the same step through the C ABI with host buffers (svm_brownian_step_io, one call per
step): H2D of the positions from pinned host memory, the step, D2H of the positions and the
energy, one synchronisation.  Per-phase CUDA events taken during the
timed steps give the dominant kernel's launch duration for `roofline`.  `cpu_baseline` times the
CPU oracle (restatement of the reference CPU path, one core as the reference's vertex-model loops
are serial) on a bounded sample of the same workload from the same equilibrated state.

reference: the CPU restatement of the reference path on all host cores (one independent replica
per core, since the reference's vertex-model loops are serial), each bench step one timestep of
every replica.  Under torchrun only rank 0 runs it.

N > 1 GPUs: independent replicas, one per GPU (scaling "weak"); a barrier and the max over ranks
of the timed region, value = all vertex-steps / that time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 100_000
PARAMS = dict(a0=1.0, p0=3.8, kr=1.0, T=0.01, mu=1.0, dt=0.01, t1=0.04)
SEED = 1137
BD_SEED = 4242
BATCH_SEED = 5150
FIRE_SEED = 9100
WORKLOAD = ("spherical vertex model, overdamped Brownian step, FP64 plain form, N=100000 cells "
            "(199996 vertices), A0=1 P0=3.8 KA=KP=1 T=0.01 mu=1 dt=0.01 T1 threshold 0.04, "
            "seeded Voronoi start")
METRIC = "vertex-steps/s at N=100k (FP64 Brownian step)"
UNIT = "vertex-steps/s"


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def job_throughput(pg, local_seconds: float, units_per_step: int, steps: int, world: int):
    """Whole-job throughput of `world` ranks that each processed units_per_step x steps units:
    the slowest rank's time (max over ranks) and all units / that time."""
    t = float(local_seconds)
    if pg is not None:
        import torch
        x = torch.tensor([t], dtype=torch.float64)
        pg.all_reduce(x, op=pg.ReduceOp.MAX)
        t = float(x.item())
    return t, world * units_per_step * steps / t


# --------------------------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{gpu_index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------------------------
def algorithmic_bytes_force(nv: int, nc: int) -> int:
    """Compulsory bytes of one launch of the fused force + Brownian + move kernel, each array it
    reads or writes counted once: positions in (24 B) and out (24 B), forces out (24 B), the
    vertex's spherical coordinates (32 B), vertex->cell, ring-predecessor and ring-successor slots
    (3 x 12 B), and per cell centroid (24 B), its spherical coordinates (32 B), (A, P) (16 B) and
    (A0, P0) (16 B)."""
    return nv * (24 + 24 + 24 + 32 + 36) + nc * (24 + 32 + 16 + 16)


def algorithmic_bytes_step(nv: int) -> int:
    """Compulsory bytes of one Brownian step (positions r/w 48, vertex->cell 12, vertex->vertex
    12, rings 12, ring sizes 2, (A0, P0) 8) = 94 B per vertex-step."""
    return 94 * nv


# From an ncu --set full capture of k_force_bd at N = 1M cells (the profiling case of this package,
# --cells 1000000 --stab 2 --steps 1): DRAM bytes read + written per vertex by one launch, and the
# FP64 pipe's busy fraction in that kernel.
FORCE_BD_DRAM_BYTES_PER_VERTEX = (1.247151e9 + 0.124883e9) / 1_999_996
FORCE_BD_FP64_PIPE_PCT = 83.4
# FP64 arithmetic thread operations (DMUL + DFMA + DADD) per vertex in one k_force_bd launch (ncu
# at N = 100k), and the FP64 issue rate they are bound by: 16 SM cycles per FP64 warp instruction
# (ncu: sm__pipe_fp64_cycles_active / sm__inst_executed_pipe_fp64 in every FP64 kernel), i.e. two
# lanes per clock on each of the 152 SMs at the 2070 MHz maximum SM clock.
FORCE_BD_FP64_OPS_PER_VERTEX = 1420
FP64_LANES_PER_CLOCK_PER_SM = 2
GB300_SMS = 152
SM_MAX_MHZ = 2070


def fp64_roofline(avg_launch_ms: float, nv: int) -> dict:
    """The force kernel against the FP64 issue rate: achieved and peak in G thread-ops/s."""
    achieved = FORCE_BD_FP64_OPS_PER_VERTEX * nv / (avg_launch_ms * 1e-3) / 1e9
    peak = GB300_SMS * FP64_LANES_PER_CLOCK_PER_SM * SM_MAX_MHZ * 1e6 / 1e9
    return {"unit": "G FP64 thread-ops/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "ops_per_vertex_ncu": FORCE_BD_FP64_OPS_PER_VERTEX,
            "peak_basis": "152 SMs x 2 FP64 lanes/clock x 2070 MHz (16 cycles per FP64 warp instruction, ncu)"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline_sample(state, steps: int):
    """The CPU oracle on one core, `steps` Brownian steps of the same workload from `state`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build_oracle()
    m = oracle.OracleModel(state["pos"], state["rings"], state["counts"], state["vcells"], state["vnbrs"],
                           state["radius"])
    m.set_preferred(PARAMS["a0"], PARAMS["p0"])
    m.set_kr(PARAMS["kr"])
    m.set_t1_threshold(PARAMS["t1"])
    noise = oracle.OracleNoise(BD_SEED)
    m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])  # warm caches
    t0 = time.perf_counter()
    for _ in range(steps):
        m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])
    dt = time.perf_counter() - t0
    nv = state["pos"].shape[0]
    return nv * steps / dt, dt


# --------------------------------------------------------------------------------------------
def run_ours(args):
    rank, world, local = dist_env()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    import numpy as np
    import torch
    import curvedspacevertexmodel_gb300 as svm
    from curvedspacevertexmodel_gb300 import _lib
    import ctypes as C

    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    torch.cuda.set_device(0)
    n = args.cells
    noise = svm.noiseSource()
    noise.setReproducibleSeed(SEED + rank)
    model = svm.sphericalVertexModel(n, noise, PARAMS["a0"], PARAMS["p0"])
    # every timing event goes on the stream the model's kernels are launched on
    stream = torch.cuda.ExternalStream(model.streamHandle())
    model.setScalarModelParameter(PARAMS["kr"])
    model.setT1Threshold(PARAMS["t1"])
    nv, nc = model.nVertices, model.nCells
    bd = svm.brownianDynamics()
    bd.setModel(model)
    bd.setT(PARAMS["T"])
    bd.setDeltaT(PARAMS["dt"])
    bd.mu = PARAMS["mu"]
    bd.noise.setReproducibleSeed(BD_SEED + rank)
    # untimed preparation: stabilisation at T = 0, P0 = 1, then equilibration at the run parameters
    bd.setT(0.0)
    model.setPreferredParameters(PARAMS["a0"], 1.0)
    bd.run(args.stab)
    bd.setT(PARAMS["T"])
    model.setPreferredParameters(PARAMS["a0"], PARAMS["p0"])
    bd.run(args.equil)
    for _ in range(max(3, args.warmup)):
        bd.integrateEquationOfMotion()
    torch.cuda.synchronize()
    model.t1Stats()
    model.fallbackCount()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")  # > L2 (129 MB)

    # ---- timed region: K steps, each after an L2 flush, events on the model's stream ----
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    _lib.call("svm_model_profile", model.handle, 1)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            starts[i].record(stream)
            bd.integrateEquationOfMotion()
            ends[i].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if pg:
        pg.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = np.zeros(_lib_phase_count(), dtype=np.float64)
    launches = np.zeros(_lib_phase_count(), dtype=np.int32)
    _lib.call("svm_model_profile_read", model.handle, ms, launches)
    t1stats = model.t1Stats()
    fallbacks_timed = model.fallbackCount()
    _lib.call("svm_model_profile", model.handle, 0)
    total_s, value = job_throughput(pg, float(sum(step_ms)) / 1e3, nv, args.steps, world)
    total_ms = 1e3 * total_s
    ms_per_step = total_ms / args.steps

    # warm-L2 reference point: K back-to-back steps in one captured run
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    bd.run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    warm_ms = e0.elapsed_time(e1) / args.steps

    # ---- e2e through the C ABI with pinned host buffers ----
    host_pos = torch.empty(3 * nv, dtype=torch.float64).pin_memory().numpy()
    host_out = torch.empty(3 * nv, dtype=torch.float64).pin_memory().numpy()
    host_pos[:] = model.returnPositions().reshape(-1)
    energy = C.c_double()
    for _ in range(args.warmup):  # untimed, as for the device-resident steps
        _lib.call("svm_brownian_step_io", model.handle, PARAMS["T"], PARAMS["dt"], PARAMS["mu"], BD_SEED + rank,
                  host_pos, host_out, C.byref(energy))
        host_pos, host_out = host_out, host_pos
    model.fallbackCount()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.call("svm_brownian_step_io", model.handle, PARAMS["T"], PARAMS["dt"], PARAMS["mu"], BD_SEED + rank,
                  host_pos, host_out, C.byref(energy))
        host_pos, host_out = host_out, host_pos
    e2e_s, e2e_value = job_throughput(pg, time.perf_counter() - t0, nv, args.steps, world)
    fallbacks_e2e = model.fallbackCount()

    status = model.deviceStatus()
    model.computeGeometry()
    energy_per_cell = model.computeEnergy() / nc
    cpu_state = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_state = dict(pos=model.returnPositions(), radius=model.radius)
        cpu_state["rings"], cpu_state["counts"] = model.rings()
        cpu_state["vcells"], cpu_state["vnbrs"] = model.vertexCellNeighbors(), model.vertexNeighbors()
    mixed = None if args.no_mixed else time_mixed_form(args, model, bd, stream, flush, nv, nc)
    batched = None if args.no_batch else time_batched_replicas(args, rank)
    fire = None if args.no_fire else time_fire(args, rank)
    if rank != 0:
        return
    # ---- roofline of the dominant kernel ----
    names = _lib.PHASES
    dom = int(np.argmax(ms))
    avg_launch_ms = ms[dom] / max(1, launches[dom])  # the force phase is one kernel per bracket
    peak, peak_kind = peaks()
    if names[dom] == "force":
        alg = algorithmic_bytes_force(nv, nc)
    else:
        alg = algorithmic_bytes_step(nv)
    achieved = alg / (avg_launch_ms / 1e3) / 1e9
    traffic = FORCE_BD_DRAM_BYTES_PER_VERTEX * nv if names[dom] == "force" else None
    cpu = None
    if cpu_state is not None:
        v, secs = cpu_baseline_sample(cpu_state, args.cpu_steps)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{args.cpu_steps} Brownian steps of the same N=100k workload from the same equilibrated "
                         f"state on one host core ({secs:.1f} s), the reference's serial CPU path restated"}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cell centres, reference init recipe)",
        "config": {"workload": WORKLOAD, "n_cells": nc, "n_vertices": nv, "stabilisation_steps": args.stab,
                   "equilibration_steps": args.equil,
                   "l2": "flushed before every timed step (512 MB write); state is ~40 MB < 129 MB L2",
                   "parallelism": f"replicas x{world}" if world > 1 else "single sphere, one GPU",
                   "noise": "in-kernel Philox4x32-10"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 24 * nv, "d2h_bytes_per_step": 24 * nv + 8,
                "area_fallback_steps": fallbacks_e2e},
        # steps whose total-area check failed (a near-degenerate corner's angle wrapped by 2 pi) and
        # recomputed every area with the triangle fan, as the reference's CPU path does (~0.3 ms each)
        "area_fallback_steps": fallbacks_timed,
        "gpu_launches": int(launches.sum()),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_force_bd" if names[dom] == "force" else f"k_{names[dom]}",
                     "peak_source": peak_kind,
                     "fp64_pipe_busy_pct_ncu": FORCE_BD_FP64_PIPE_PCT,
                     "fp64": fp64_roofline(avg_launch_ms, nv) if names[dom] == "force" else None,
                     "note": "FP64-pipe bound (ncu: FP64 pipe 83% busy, DRAM 3%); HBM fraction is small by construction",
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_launch_ms},
        "phases_ms_per_step": {nm: float(t / args.steps) for nm, t in zip(names, ms)},
        "warm_l2_ms_per_step": warm_ms,
        "t1_per_step": {k: v / args.steps for k, v in t1stats.items()},
        "wall_s": wall,
        "device_status": status,
        "energy_per_cell": energy_per_cell,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "mixed_form": mixed,
        "batched_replicas": batched,
        "fire_warm_start": fire,
    }
    print(json.dumps(out), flush=True)


def time_fire(args, rank):
    """FIRE to max|F| < 1e-9 at N = 20k cells, learned warm start against plain FIRE, on held-out
    instances (P0 uniform in [3.6, 3.8], seeds not used in training).  Start states: stabilisation
    then 500 Brownian steps at T = 0.01; FIRE dt0 0.01, alpha0 0.1, dtMax 0.1, finc 1.1, fdec 0.5,
    alphaDec 0.9, NMin 5; FP64 vector-form forces; T1 on.  Wall time of each minimisation,
    synchronised on both sides; the warm time includes the network's inference, the step-length
    choice and any fallback."""
    import numpy as np
    from curvedspacevertexmodel_gb300 import warm_start as ws
    net = ws.load(os.path.join(ROOT, "curvedspacevertexmodel_gb300", "data", "warm_start_n20k.npz"))
    rng = np.random.default_rng(FIRE_SEED + rank)
    rows = [ws.compare(net, 20000, float(p0), FIRE_SEED + 100 * rank + i)
            for i, p0 in enumerate(rng.uniform(3.6, 3.8, args.fire_instances))]
    net.close()
    plain = sum(r["plain_s"] for r in rows)
    warm = sum(r["warm_s"] for r in rows)
    return {"metric": "FIRE wall time to max|F| < 1e-9, warm start / plain", "value": warm / plain,
            "unit": "ratio (lower is better)", "plain_s": plain, "warm_s": warm,
            "plain_ms_per_iteration": 1e3 * plain / sum(r["plain_iterations"] for r in rows),
            "instances": [{k: r[k] for k in ("p0", "seed", "plain_s", "plain_iterations", "warm_s", "warm_iterations",
                                             "fallback", "warm_step_length", "energy_start", "energy_after_warm_start",
                                             "energy_per_cell_plain", "energy_per_cell_warm")} for r in rows],
            "workload": "N=20000, P0 U[3.6, 3.8], start = stabilisation + 500 Brownian steps at T=0.01, "
                        "FIRE dt0 0.01 alpha0 0.1 dtMax 0.1 finc 1.1 fdec 0.5, FP64 vector-form forces, T1 on"}


def time_batched_replicas(args, rank):
    """Batched replicas: 512 independent spheres, N per replica log-uniform in [100, 5000] cells,
    P0 uniform in [3.6, 3.95], T log-uniform in [1e-4, 1e-1], dt = 0.01, T1 threshold 0.04,
    mixed-precision form, all replicas in each launch and the steps replayed from a captured
    graph; block sizes from the autotuner.  Prepared like the single sphere (100 steps at T = 0,
    P0 = 1, then 100 steps at the run parameters).  The state (~150 MB) exceeds L2, so no flush."""
    import numpy as np
    import torch
    import curvedspacevertexmodel_gb300 as svm
    rng = np.random.default_rng(BATCH_SEED + rank)
    n_rep = args.replicas
    sizes = np.exp(rng.uniform(np.log(100), np.log(5000), n_rep)).astype(int)
    p0s = rng.uniform(3.6, 3.95, n_rep)
    temps = np.exp(rng.uniform(np.log(1e-4), np.log(1e-1), n_rep))
    seeds = BATCH_SEED + 1000 * (rank + 1) + np.arange(n_rep)
    t0 = time.perf_counter()
    b = svm.sphericalVertexModelBatch(sizes, seeds, p0=1.0)
    setup_s = time.perf_counter() - t0
    b.setT1Threshold(PARAMS["t1"])
    bd = svm.brownianDynamics()
    bd.setModel(b)
    bd.setDeltaT(PARAMS["dt"])
    bd.noise.setReproducibleSeed(BATCH_SEED + 7 + rank)
    b.setTemperatures(np.zeros(n_rep))
    bd.run(100)
    b.setPreferredParameters(1.0, p0s)
    b.setTemperatures(temps)
    b.autotune(64, 1024, 64, 3, 100000)
    bd.run(100)  # tuner sampling (steps run one by one) + equilibration
    bd.run(args.steps)  # graph capture outside the timed region
    stream = torch.cuda.ExternalStream(b.streamHandle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b.t1Stats()
    torch.cuda.synchronize()
    e0.record(stream)
    bd.run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    t1 = b.t1Stats()
    b.computeGeometry()
    e = b.replicaEnergies() / sizes
    _, _, taken = b.replicaAreaCheck()
    out = {"workload": f"{n_rep} replicas, N log-uniform [100, 5000] cells (total {int(sizes.sum())} cells, "
                       f"{b.nVertices} vertices), P0 U[3.6, 3.95], T logU[1e-4, 1e-1], dt 0.01, mixed form, T1 on",
           "seed": BATCH_SEED, "ms_per_step": ms, "value": b.nVertices / (ms / 1e3), "unit": UNIT,
           "block_sizes": b.blockSizes(), "t1_per_step": {k: v / args.steps for k, v in t1.items()},
           "energy_per_cell_min_median_max": [float(e.min()), float(np.median(e)), float(e.max())],
           "area_fallback_replicas": int(taken.sum()), "device_status": b.deviceStatus(),
           "setup_s": setup_s, "l2": "state ~150 MB > 129 MB L2; steps back to back from one graph"}
    b.close()
    return out


def algorithmic_bytes_force_mixed(nv: int, nc: int) -> int:
    """Compulsory bytes of one launch of the mixed-form force + Brownian + move kernel: FP32
    positions in and out and forces out (3 x 16 B), the three slot triples (36 B), and per cell the
    FP32 centroid (16 B), (A, P) (16 B) and (A0, P0) (16 B)."""
    return nv * (16 * 3 + 36) + nc * (16 + 16 + 16)


def time_mixed_form(args, model, bd, stream, flush, nv, nc):
    """The same step in the mixed-precision form (FP32 positions, forces and integration; FP64
    included angles, areas, energy and renormalisation) from the same equilibrated state, timed the
    same way.  A secondary line: the headline metric is the FP64 form."""
    import numpy as np
    import torch
    from curvedspacevertexmodel_gb300 import _lib
    model.precision = "mixed"
    for _ in range(max(3, args.warmup)):
        bd.integrateEquationOfMotion()
    torch.cuda.synchronize()
    model.t1Stats()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    _lib.call("svm_model_profile", model.handle, 1)
    torch.cuda.synchronize()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        starts[i].record(stream)
        bd.integrateEquationOfMotion()
        ends[i].record(stream)
    torch.cuda.synchronize()
    ms = np.zeros(len(_lib.PHASES), dtype=np.float64)
    launches = np.zeros(len(_lib.PHASES), dtype=np.int32)
    _lib.call("svm_model_profile_read", model.handle, ms, launches)
    _lib.call("svm_model_profile", model.handle, 0)
    t1 = model.t1Stats()
    total_ms = float(sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
    status = model.deviceStatus()
    model.computeGeometry()
    e = model.computeEnergy() / nc
    _, _, fallback = model.areaCheck()
    model.precision = "fp64"
    fi = _lib.PHASES.index("force")
    force_ms = ms[fi] / max(1, launches[fi])
    alg = algorithmic_bytes_force_mixed(nv, nc)
    peak, peak_kind = peaks()
    return {"ms_per_step": total_ms / args.steps, "value": nv * args.steps / (total_ms / 1e3), "unit": UNIT,
            "phases_ms_per_step": {nm: float(t / args.steps) for nm, t in zip(_lib.PHASES, ms)},
            "force_kernel": {"kernel": "k32_force_bd", "avg_launch_ms": force_ms, "algorithmic_bytes_per_launch": alg,
                             "achieved_gbs": alg / (force_ms / 1e3) / 1e9,
                             "frac_of_" + peak_kind + "_hbm": alg / (force_ms / 1e3) / 1e9 / peak},
            "t1_per_step": {k: v / args.steps for k, v in t1.items()},
            "energy_per_cell": e, "area_fallback_taken": bool(fallback), "device_status": status,
            "gpu_launches": int(launches.sum())}


def _lib_phase_count():
    from curvedspacevertexmodel_gb300 import _lib
    return len(_lib.PHASES)


# --------------------------------------------------------------------------------------------
def _ref_worker(idx, n, steps, warmup, stab, barrier, q):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    import topology as otopo
    pts = oracle.OracleNoise(SEED + idx).cell_centres(n)
    t = otopo.topology(pts)
    m = oracle.OracleModel(t["pos"], t["rings"], t["counts"], t["vcells"], t["vnbrs"], math.sqrt(n / (4 * math.pi)))
    m.set_preferred(PARAMS["a0"], PARAMS["p0"])
    m.set_kr(PARAMS["kr"])
    m.set_t1_threshold(PARAMS["t1"])
    noise = oracle.OracleNoise(BD_SEED + idx)
    m.set_preferred(PARAMS["a0"], 1.0)  # the reference driver's stabilisation (sphericalVertex.cpp:106-115)
    for _ in range(stab):
        m.brownian_step(noise, 0.0, PARAMS["dt"], PARAMS["mu"])
    m.set_preferred(PARAMS["a0"], PARAMS["p0"])
    for _ in range(warmup):
        m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])
    barrier.wait()
    for _ in range(steps):
        m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])
        barrier.wait()
    q.put(int(np.asarray(m.positions()).shape[0]))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build_oracle()
    cores = args.ref_cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores + 1)
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(i, args.cells, args.steps, args.warmup, args.ref_stab, barrier, q))
             for i in range(cores)]
    for p in procs:
        p.start()
    barrier.wait()  # all replicas built and warmed up
    t0 = time.perf_counter()
    for _ in range(args.steps):
        barrier.wait()
    dt = time.perf_counter() - t0
    nvs = [q.get() for _ in procs]
    for p in procs:
        p.join()
    value = sum(nvs) * args.steps / dt
    sample = (f"{cores} independent replicas (one per host core) of the N=100k workload, each bench step one "
              f"Brownian timestep of every replica; CPU restatement of the reference path (-O3)")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cell centres, reference init recipe)",
        "config": {"workload": WORKLOAD, "n_cells": args.cells, "n_vertices": nvs[0] if nvs else None,
                   "parallelism": f"{cores} host processes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--cells", type=int, default=N_CELLS)
    ap.add_argument("--stab", type=int, default=100, help="untimed stabilisation steps (T=0, P0=1)")
    ap.add_argument("--equil", type=int, default=200, help="untimed equilibration steps before warm-up")
    ap.add_argument("--cpu-steps", type=int, default=25, help="steps of the one-core CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision form's secondary timing")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-replica secondary timing")
    ap.add_argument("--replicas", type=int, default=512)
    ap.add_argument("--no-fire", action="store_true", help="skip the FIRE warm-start comparison")
    ap.add_argument("--fire-instances", type=int, default=2)
    ap.add_argument("--ref-cores", type=int, default=0)
    ap.add_argument("--ref-stab", type=int, default=30, help="stabilisation steps of each reference replica")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
