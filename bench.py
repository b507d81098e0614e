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

Other workloads (off by default, one JSON line each; --mode):
  forms    the FP64 plain form against the FP32-bulk/FP64-area form over --steps (default 10,000)
           steps at N = 100k with the same injected noise: energy, area and perimeter errors, T1-set
           agreement, time-averaged energies with their standard errors, and each form's GB/s;
  large    N = 1M cells: --steps (default 5,000) mixed-form Brownian steps with the HBM fraction of
           the step, then FIRE to max|F| < 1e-8, plain and from the learned warm start;
  batch    512 replicas for --steps (default 10,000) batched steps, and per-replica energy errors of
           a 32-replica subset against FP64 single-sphere runs (same state, and time averages);
  profile  a small untimed run for profilers (ncu -k ...): --cells, --stab, --steps, --equil and
           the options --mixed, --replicas, --fire, --neighbors, --sub-grid, --active, --dynamics;
  fire-ablation  where FIRE's iterations go at N = 20k, and how many remain from the minimum
           itself after a few thermal steps (the bound on any warm start).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
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


def config_of(args, n_vertices, parallelism):
    """The workload's config, the same for both arms except `parallelism`."""
    return {"workload": WORKLOAD, "n_cells": args.cells, "n_vertices": n_vertices,
            "stabilisation_steps": args.stab, "equilibration_steps": args.equil,
            "l2": "GPU arm: flushed before every timed step (512 MB write); state is ~40 MB < 129 MB L2",
            "parallelism": parallelism}


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
        self.dir = tempfile.mkdtemp(prefix="svm_bench_clocks_")
        self.path = os.path.join(self.dir, f"clocks_rank{gpu_index}.csv")

    def __enter__(self):
        try:
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
        import shutil
        shutil.rmtree(self.dir, ignore_errors=True)
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


# From an ncu --set full capture of one k_force_bd launch at N = 100k cells (bench.py --mode profile
# --cells 100000 --stab 2 --steps 1; profiles/k_force_bd_n100k_full.md): DRAM bytes read + written
# per vertex by one launch, and the FP64 and integer (ALU) pipes' busy fractions in that kernel.
FORCE_BD_DRAM_BYTES_PER_VERTEX = (32.27776e6 + 0.608512e6) / 199_996
FORCE_BD_FP64_PIPE_PCT = 67.7
FORCE_BD_ALU_PIPE_PCT = 27.7
# FP64 arithmetic thread operations (DMUL + DFMA + DADD) per vertex in one k_force_bd launch of the
# build whose divisions and square roots are the hardware sequences (ncu at N = 100k), and the FP64
# issue rate they are bound by: 16 SM cycles per FP64 warp instruction (ncu:
# sm__pipe_fp64_cycles_active / sm__inst_executed_pipe_fp64 in every FP64 kernel), i.e. two lanes
# per clock on each of the 152 SMs at the 2070 MHz maximum SM clock.  The default build computes the
# divisions and square roots, and the products that start the gradients' dependency chains, on the
# integer pipes (same results), so the rate below is FP64-pipe-equivalent work: above 1 it does that
# work faster than the FP64 pipe alone could issue it.
FORCE_BD_FP64_OPS_PER_VERTEX = 1420
FP64_LANES_PER_CLOCK_PER_SM = 2
GB300_SMS = 152
SM_MAX_MHZ = 2070


def fp64_roofline(avg_launch_ms: float, nv: int) -> dict:
    """The force kernel against the FP64 issue rate: the hardware-division build's FP64 instructions
    per vertex over the measured launch (FP64-pipe-equivalent work), and the peak, in G thread-ops/s."""
    achieved = FORCE_BD_FP64_OPS_PER_VERTEX * nv / (avg_launch_ms * 1e-3) / 1e9
    peak = GB300_SMS * FP64_LANES_PER_CLOCK_PER_SM * SM_MAX_MHZ * 1e6 / 1e9
    return {"unit": "G FP64 thread-ops/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "ops_per_vertex_ncu": FORCE_BD_FP64_OPS_PER_VERTEX,
            "peak_basis": "152 SMs x 2 FP64 lanes/clock x 2070 MHz (16 cycles per FP64 warp instruction, ncu)",
            "work_basis": "FP64 instructions per vertex of the build with hardware divisions and square roots; "
                          "the measured build computes those on the integer pipes (bit-identical results)"}


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
def rank_visible_devices(local: int, visible):
    """CUDA_VISIBLE_DEVICES for local rank `local`: its own entry of an inherited device list (a
    launcher may export every GPU of the node), else the device with the rank's number."""
    devs = [d.strip() for d in visible.split(",") if d.strip()] if visible else []
    return devs[local % len(devs)] if devs else str(local)


def run_ours(args):
    rank, world, local = dist_env()
    if world > 1:  # one GPU per rank, seen by the rank as device 0
        os.environ["CUDA_VISIBLE_DEVICES"] = rank_visible_devices(local, os.environ.get("CUDA_VISIBLE_DEVICES"))
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
    _lib.call("svm_model_profile", model.handle, force_only_mask())  # the force kernel's events only
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
    phases = phase_breakdown(model, bd, stream, flush, args.steps)
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
                         f"state on one host core ({secs:.1f} s), the reference's serial CPU path restated (bit for "
                         f"bit the reference build's trajectory; the build runs {PORT_TIME_OVER_REFERENCE_BUILD}x "
                         f"faster per step on an x86-64 core)"}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cell centres, reference init recipe)",
        "config": config_of(args, nv, f"replicas x{world}" if world > 1 else "single sphere, one GPU"),
        "noise": "in-kernel Philox4x32-10 with ziggurat normals",
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
                     "alu_pipe_busy_pct_ncu": FORCE_BD_ALU_PIPE_PCT,
                     "fp64": fp64_roofline(avg_launch_ms, nv) if names[dom] == "force" else None,
                     "note": "FP64-issue and latency bound (ncu: FP64 pipe 68% and integer pipes 28% busy, DRAM "
                             "under 1%; divisions, square roots and chain-starting products on the integer "
                             "pipes); HBM fraction is small by construction",
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_launch_ms},
        "phases_ms_per_step": phases,
        "phases_note": "every phase bracketed by events, over as many further steps after the timed region",
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


def force_only_mask():
    from curvedspacevertexmodel_gb300 import _lib
    return _lib.SVM_PROFILE_ONLY | (1 << _lib.PHASES.index("force"))


def phase_breakdown(model, bd, stream, flush, steps):
    """Milliseconds per step of every phase, from `steps` further steps (each after the L2 flush)
    with every phase bracketed by events -- outside the timed region, whose steps carry only the
    force kernel's pair of events (a pair per phase adds ~20 us to a step)."""
    import numpy as np
    import torch
    from curvedspacevertexmodel_gb300 import _lib
    ms = np.zeros(len(_lib.PHASES), dtype=np.float64)
    launches = np.zeros(len(_lib.PHASES), dtype=np.int32)
    _lib.call("svm_model_profile", model.handle, 1)
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        bd.integrateEquationOfMotion()
    torch.cuda.synchronize()
    _lib.call("svm_model_profile_read", model.handle, ms, launches)
    _lib.call("svm_model_profile", model.handle, 0)
    return {nm: float(t / steps) for nm, t in zip(_lib.PHASES, ms)}


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
    _lib.call("svm_model_profile", model.handle, force_only_mask())
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
    phases = phase_breakdown(model, bd, stream, flush, args.steps)
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
            "phases_ms_per_step": phases,
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
# The CPU restatement of the reference path (oracle/, bit for bit the reference's own build on the
# same inputs) against that build, on one core of an x86-64 host, timed in lockstep on the identical
# N = 20k trajectory (the build cannot run here: it is compiled from the reference's sources, which
# only the development host has): the restatement takes 1.15x the reference build's time per step.
PORT_TIME_OVER_REFERENCE_BUILD = 1.15


def _ref_worker(idx, n, steps, warmup, stab, equil, barrier, q):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    import topology as otopo
    pts = oracle.OracleNoise(SEED + idx).cell_centres(n)
    t = otopo.topology(pts)
    m = oracle.OracleModel(t["pos"], t["rings"], t["counts"], t["vcells"], t["vnbrs"], math.sqrt(n / (4 * math.pi)))
    m.set_kr(PARAMS["kr"])
    m.set_t1_threshold(PARAMS["t1"])
    noise = oracle.OracleNoise(BD_SEED + idx)
    # the preparation of the GPU arm (the reference driver's, sphericalVertex.cpp:104-125): stab steps
    # at T = 0 with P0 = 1, then equil steps at the run parameters, then the warm-up steps
    m.set_preferred(PARAMS["a0"], 1.0)
    for _ in range(stab):
        m.brownian_step(noise, 0.0, PARAMS["dt"], PARAMS["mu"])
    m.set_preferred(PARAMS["a0"], PARAMS["p0"])
    for _ in range(equil + warmup):
        m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])
    f0 = m.fallback_count()
    barrier.wait()
    for _ in range(steps):
        m.brownian_step(noise, PARAMS["T"], PARAMS["dt"], PARAMS["mu"])
        barrier.wait()
    q.put((int(np.asarray(m.positions()).shape[0]), m.fallback_count() - f0))


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
    procs = [ctx.Process(target=_ref_worker, args=(i, args.cells, args.steps, args.warmup, args.stab, args.equil,
                                                   barrier, q))
             for i in range(cores)]
    for p in procs:
        p.start()
    barrier.wait()  # all replicas built, prepared and warmed up
    t0 = time.perf_counter()
    for _ in range(args.steps):
        barrier.wait()
    dt = time.perf_counter() - t0
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
    nvs = [r[0] for r in res]
    value = sum(nvs) * args.steps / dt
    sample = (f"{cores} independent replicas (one per host core) of the N=100k workload, each prepared as the GPU "
              f"arm ({args.stab} stabilisation + {args.equil} equilibration steps), each bench step one Brownian "
              f"timestep of every replica; CPU restatement of the reference path (-O3), bit for bit the reference "
              f"build's trajectory, which runs {PORT_TIME_OVER_REFERENCE_BUILD}x faster per step on an x86-64 core")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded cell centres, reference init recipe)",
        "config": config_of(args, nvs[0] if nvs else None, f"{cores} host processes"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "area_fallback_steps": int(sum(r[1] for r in res)),
        "area_fallback_note": "replica-steps of the timed region whose total-area check took the triangle fan",
        "port_time_over_reference_build": PORT_TIME_OVER_REFERENCE_BUILD,
        "value_at_reference_build_speed": value * PORT_TIME_OVER_REFERENCE_BUILD,
    }
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------------------------
# Other workloads (--mode): each prints one JSON line.

def _prepared_model(svm, n, seed, stab, equil, p0=PARAMS["p0"], T=PARAMS["T"]):
    """A seeded model prepared with the reference driver's recipe: stab steps at T = 0 with P0 = 1,
    then equil graph-replayed steps at (P0, T)."""
    noise = svm.noiseSource()
    noise.setReproducibleSeed(seed)
    m = svm.sphericalVertexModel(n, noise, PARAMS["a0"], p0)
    m.setT1Threshold(PARAMS["t1"])
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.setDeltaT(PARAMS["dt"])
    bd.noise.setReproducibleSeed(seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(PARAMS["a0"], 1.0)
    if stab:
        bd.run(stab)
    bd.setT(T)
    m.setPreferredParameters(PARAMS["a0"], p0)
    if equil:
        bd.run(equil)
    return m, bd


def _timed_run(m, bd, steps):
    """Milliseconds per step of `steps` graph-replayed steps, CUDA events on the model's stream."""
    import torch
    stream = torch.cuda.ExternalStream(m.streamHandle())
    bd.run(steps)  # capture outside the timed region
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    bd.run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _mean_se(x):
    """Mean and standard error of a series of (block) averages."""
    import numpy as np
    x = np.asarray(x, dtype=np.float64)
    return float(x.mean()), float(x.std(ddof=1) / math.sqrt(len(x))) if len(x) > 1 else float("nan")


def mode_forms(args):
    """The FP64 plain form against the FP32-bulk/FP64-area form at N = 100k over args.steps steps.
    Both start from the same FP32-representable prepared state and are driven by the same host
    normals (injected each step), so they differ only by arithmetic.  At every args.every steps:
    energy per cell in each form, their relative difference, area and perimeter differences (cells
    matched by index), the fraction of vertices whose neighbours agree, and the T1 flips of the
    interval in both forms with how many coincide (same edge, same 200-step window).  The summary
    gives time-averaged energies per cell over the checkpoints after the first with their standard
    errors (the forms separate chaotically, so only statistics can be compared), and each form's
    step time and GB/s (algorithmic bytes: 94 B per vertex-step FP64, 70 B mixed) from graph-replayed
    steps timed with CUDA events."""
    import numpy as np
    import curvedspacevertexmodel_gb300 as svm
    a, _ = _prepared_model(svm, args.cells, SEED, args.stab, args.equil)
    st = a.saveState()
    st["pos"] = st["pos"].astype(np.float32).astype(np.float64)
    a.loadState(st)
    nb = svm.noiseSource()
    nb.setReproducibleSeed(SEED)
    b = svm.sphericalVertexModel(args.cells, nb, radius=a.radius)
    b.setT1Threshold(PARAMS["t1"])
    b.loadState(st)
    b.setPreferredParameters(PARAMS["a0"], PARAMS["p0"])
    b.precision = "mixed"
    bda, bdb = svm.brownianDynamics(), svm.brownianDynamics()
    for bd, m in ((bda, a), (bdb, b)):
        bd.setModel(m)
        bd.setT(PARAMS["T"])
        bd.setDeltaT(PARAMS["dt"])
    rng = np.random.default_rng(SEED + 7)
    a.takeFlips()
    b.takeFlips()
    nfa = nfb = ncommon = 0
    rows = []
    for step in range(1, args.steps + 1):
        xi = rng.standard_normal((a.nVertices, 3))
        for bd in (bda, bdb):
            bd.injectNoise(xi)
            bd.integrateEquationOfMotion()
        if step % 200 == 0 or step % args.every == 0:  # the flip logs hold 65,536 flips
            fa, fb = a.takeFlips(), b.takeFlips()
            nfa += len(fa)
            nfb += len(fb)
            ncommon += len(set(map(tuple, fa)) & set(map(tuple, fb)))
        if step % args.every == 0:
            a.computeGeometry()
            b.computeGeometry()
            ea, eb = a.computeEnergy() / a.nCells, b.computeEnergy() / b.nCells
            apa, apb = a.areaPerimeter(), b.areaPerimeter()
            same_nb = np.mean(np.all(np.sort(a.vertexNeighbors(), 1) == np.sort(b.vertexNeighbors(), 1), 1))
            rows.append({"step": step, "energy_per_cell_fp64": ea, "energy_per_cell_mixed": eb,
                         "energy_rel_diff": abs(ea - eb) / ea,
                         "area_abs_diff_median_max": [float(np.median(np.abs(apa[:, 0] - apb[:, 0]))),
                                                      float(np.max(np.abs(apa[:, 0] - apb[:, 0])))],
                         "perimeter_abs_diff_median_max": [float(np.median(np.abs(apa[:, 1] - apb[:, 1]))),
                                                           float(np.max(np.abs(apa[:, 1] - apb[:, 1])))],
                         "same_neighbour_fraction": float(same_nb), "flips_fp64": nfa, "flips_mixed": nfb,
                         "flips_common": ncommon})
            nfa = nfb = ncommon = 0
    peak, peak_kind = peaks()
    ms64 = _timed_run(a, bda, 50)
    ms32 = _timed_run(b, bdb, 50)
    later = rows[1:] if len(rows) > 2 else rows
    m64, se64 = _mean_se([r["energy_per_cell_fp64"] for r in later])
    m32, se32 = _mean_se([r["energy_per_cell_mixed"] for r in later])
    nv = a.nVertices
    out = {"mode": "forms", "workload": f"N={args.cells}, FP64 plain vs FP32-bulk/FP64-area, {args.steps} steps, "
                                        f"same injected normals, A0=1 P0=3.8 T=0.01 dt=0.01 T1 0.04",
           "checkpoints": rows,
           "time_averaged_energy_per_cell": {"fp64": [m64, se64], "mixed": [m32, se32],
                                             "difference_over_combined_se": abs(m64 - m32) / math.hypot(se64, se32),
                                             "relative_difference": abs(m64 - m32) / m64,
                                             "over": f"checkpoints {later[0]['step']}..{later[-1]['step']}"},
           "flips_total": {"fp64": sum(r["flips_fp64"] for r in rows), "mixed": sum(r["flips_mixed"] for r in rows),
                           "common": sum(r["flips_common"] for r in rows)},
           "step_time": {"fp64_ms": ms64, "mixed_ms": ms32,
                         "fp64_gbs": 94 * nv / (ms64 * 1e-3) / 1e9, "mixed_gbs": 70 * nv / (ms32 * 1e-3) / 1e9,
                         "fp64_frac_of_" + peak_kind + "_hbm": 94 * nv / (ms64 * 1e-3) / 1e9 / peak,
                         "mixed_frac_of_" + peak_kind + "_hbm": 70 * nv / (ms32 * 1e-3) / 1e9 / peak,
                         "timing": "50 graph-replayed steps, CUDA events, warm L2"},
           "device_status": [a.deviceStatus(), b.deviceStatus()]}
    print(json.dumps(out), flush=True)


def mode_large(args):
    """N = 1,000,000 cells (1,999,996 vertices): the reference's initialisation recipe (seeded
    Voronoi start; args.stab steps at T = 0, P0 = 1), then P0 = 3.75, T = 0.005, dt = 0.01, T1
    threshold 0.04, args.steps mixed-form Brownian steps (graph-replayed, CUDA events; HBM fraction
    from the 70 B per vertex-step of the mixed form), then FIRE to max|F| < 1e-8 (FP64 vector-form
    forces, T1 on), plain and from the learned warm start (fallback to plain FIRE from the start
    when the warm start raises the energy)."""
    import numpy as np
    import torch
    import curvedspacevertexmodel_gb300 as svm
    from curvedspacevertexmodel_gb300 import _lib
    from curvedspacevertexmodel_gb300 import warm_start as ws
    out = {"mode": "large", "workload": f"N={args.cells}, P0=3.75, T=0.005, dt=0.01, T1 0.04, {args.steps} mixed-form "
                                        f"Brownian steps, then FIRE to max|F|<1e-8 (FP64 vector form, T1 on), plain "
                                        f"vs learned warm start"}
    t0 = time.perf_counter()
    m, bd = _prepared_model(svm, args.cells, SEED, args.stab, 0, p0=3.75, T=0.005)
    out["setup_s"] = time.perf_counter() - t0
    m.precision = "mixed"
    bd.run(10)
    m.t1Stats()
    stream = torch.cuda.ExternalStream(m.streamHandle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    bd.run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    peak, peak_kind = peaks()
    t1 = m.t1Stats()
    gbs = 70 * m.nVertices / (ms * 1e-3) / 1e9
    out["brownian"] = {"ms_per_step": ms, "vertex_steps_per_s": m.nVertices / (ms * 1e-3),
                       "algorithmic_gbs": gbs, "frac_of_" + peak_kind + "_hbm": gbs / peak,
                       "t1_flips_per_step": t1["flips"] / args.steps, "device_status": m.deviceStatus(),
                       "area_fallback_taken_last_step": bool(m.areaCheck()[2])}
    m.computeGeometry()
    out["brownian"]["energy_per_cell"] = m.computeEnergy() / m.nCells
    # ensemble error bars: from the same state, 10 blocks of 200 steps in each form (the FP64 form with
    # its own noise stream), the energy per cell after every block; mean and standard error of each,
    # and their difference in combined standard errors
    if args.ensemble_blocks > 0:
        state = m.saveState()
        ens = {}
        for form in ("mixed", "fp64"):
            m.precision = "fp64"   # the state goes in through the FP64 form, then the form is chosen
            m.loadState(state)
            m.precision = form
            series = []
            for _ in range(args.ensemble_blocks):
                bd.run(200)
                m.computeGeometry()
                series.append(m.computeEnergy() / m.nCells)
            ens[form] = _mean_se(series)
        (mm, sm), (mf, sf) = ens["mixed"], ens["fp64"]
        out["ensemble_energy_per_cell"] = {
            "mixed": [mm, sm], "fp64": [mf, sf], "relative_difference": (mm - mf) / mf,
            "difference_over_combined_se": (mm - mf) / max(1e-300, (sm * sm + sf * sf) ** 0.5),
            "blocks": f"{args.ensemble_blocks} blocks of 200 steps from the same state after the timed run, "
                      "energy per cell after each block"}
        m.precision = "fp64"
        m.loadState(state)
        m.precision = "mixed"
    if args.fire_cap > 0:
        m.precision = "fp64_vector"
        start = m.saveState()
        e_start = ws.energy(m)

        def fire(cap):
            f = svm.energyMinimizerFIRE(m)
            prm = list(ws.FIRE_PARAMS)
            prm[7] = 1e-8
            f.setFIREParameters(*prm)
            f.setCriterion(_lib.SVM_FIRE_MAX_FORCE)
            f.setMaximumIterations(cap)
            m.synchronize()
            ts = time.perf_counter()
            f.minimize()
            m.synchronize()
            st = f.state()
            return st["iterations"], time.perf_counter() - ts, st["max_force"]

        it, secs, fmax = fire(args.fire_cap)
        out["fire_plain"] = {"iterations": it, "seconds": secs, "max_force": fmax,
                             "converged": bool(fmax < 1e-8), "energy_per_cell": ws.energy(m) / m.nCells,
                             "ms_per_iteration": 1e3 * secs / max(1, it), "device_status": m.deviceStatus()}
        m.loadState(start)
        net = ws.load(os.path.join(ROOT, "curvedspacevertexmodel_gb300", "data", "warm_start_n20k.npz"))
        m.synchronize()
        ts = time.perf_counter()
        base = net.outputScale
        net.setOutputScale(0.25 * base)
        net.warmStart(m)
        net.setOutputScale(base)
        e_w = ws.energy(m)
        fallback = ws.fallback_reason(e_start, e_w)
        if fallback:
            m.loadState(start)
        it_w, _, fmax_w = fire(args.fire_cap)
        m.synchronize()
        out["fire_warm"] = {"iterations": it_w, "seconds": time.perf_counter() - ts, "max_force": fmax_w,
                            "converged": bool(fmax_w < 1e-8), "energy_start": e_start, "energy_after_warm_start": e_w,
                            "fallback": fallback, "energy_per_cell": ws.energy(m) / m.nCells,
                            "device_status": m.deviceStatus()}
        net.close()
    print(json.dumps(out), flush=True)


def _replica_state(b, r):
    """Replica r of a batch as a single sphere's arrays (indices renumbered from 0)."""
    import numpy as np
    cs, vs = b.cellSlice(r), b.vertexSlice(r)
    rings, counts = b.rings()
    rr = rings[cs].copy()
    rr[rr >= 0] -= vs.start
    return dict(pos=b.returnPositions()[vs], rings=rr, counts=counts[cs],
                vcells=b.vertexCellNeighbors()[vs] - cs.start, vnbrs=b.vertexNeighbors()[vs] - vs.start)


def _single_from_state(svm, st, radius, p0):
    topo = svm.Topology.from_arrays(st["pos"], st["rings"], st["counts"], st["vcells"], st["vnbrs"])
    m = svm.sphericalVertexModel(len(st["counts"]), topology=topo, a0=PARAMS["a0"], p0=p0, radius=radius)
    m.setT1Threshold(PARAMS["t1"])
    return m


def mode_batch(args):
    """512 replicas (N log-uniform in [100, 5000] cells, P0 U[3.6, 3.95], T logU[1e-4, 1e-1], dt
    0.01, mixed form, T1 on), prepared like the single sphere (args.stab steps at T = 0, P0 = 1),
    autotuned, then args.steps batched Brownian steps in graph-replayed chunks timed with CUDA events.
    Errors against FP64 for a 32-replica subset (every 16th replica):
    (1) same state: each replica's final state evaluated in FP64 as a single sphere against the
        batch's mixed-form energy of that state;
    (2) trajectories: the subset's prepared states as a batch of their own (mixed form) and as 32 FP64
        single spheres, all driven by the same injected normals for args.compare_steps steps; the
        relative energy-per-cell difference at checkpoints (the forms separate by FP32 rounding,
        amplified along the trajectory)."""
    import numpy as np
    import torch
    import curvedspacevertexmodel_gb300 as svm
    rng = np.random.default_rng(BATCH_SEED)
    n_rep = args.replicas
    sizes = np.exp(rng.uniform(np.log(100), np.log(5000), n_rep)).astype(int)
    p0s = rng.uniform(3.6, 3.95, n_rep)
    temps = np.exp(rng.uniform(np.log(1e-4), np.log(1e-1), n_rep))
    seeds = BATCH_SEED + 1000 + np.arange(n_rep)
    b = svm.sphericalVertexModelBatch(sizes, seeds, p0=1.0)
    b.setT1Threshold(PARAMS["t1"])
    bd = svm.brownianDynamics()
    bd.setModel(b)
    bd.setDeltaT(PARAMS["dt"])
    bd.noise.setReproducibleSeed(BATCH_SEED + 7)
    b.setTemperatures(np.zeros(n_rep))
    bd.run(args.stab)
    b.setPreferredParameters(PARAMS["a0"], p0s)
    b.setTemperatures(temps)
    subset = list(range(0, n_rep, max(1, n_rep // 32)))[:32]
    starts = [_replica_state(b, r) for r in subset]
    b.autotune(64, 1024, 64, 3, 100000)
    bd.run(100)  # tuner sampling; these steps count towards the run
    chunk = max(1, min(1000, (args.steps - 100) // 10))
    bd.run(chunk)  # graph capture
    n_chunks = max(1, (args.steps - 100 - chunk) // chunk)
    stream = torch.cuda.ExternalStream(b.streamHandle())
    b.t1Stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(n_chunks):
        bd.run(chunk)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / (chunk * n_chunks)
    steps_done = 100 + chunk * (n_chunks + 1)
    t1 = b.t1Stats()
    b.computeGeometry()
    final_mixed = b.replicaEnergies()
    same = []
    for r in subset:
        s1 = _single_from_state(svm, _replica_state(b, r), float(b.radii[r]), float(p0s[r]))
        s1.computeGeometry()
        e64 = s1.computeEnergy()
        same.append(abs(final_mixed[r] - e64) / abs(e64))
        s1.close()
    status = b.deviceStatus()
    nv_all = b.nVertices
    b.close()
    # (2) the subset from its prepared states: a mixed-form batch and FP64 singles, same normals
    topo = [svm.Topology.from_arrays(st["pos"], st["rings"], st["counts"], st["vcells"], st["vnbrs"]) for st in starts]
    sub = svm.sphericalVertexModelBatch(sizes[subset], seeds[subset], p0=1.0, topologies=topo)
    sub.setT1Threshold(PARAMS["t1"])
    sub.setPreferredParameters(PARAMS["a0"], p0s[subset])
    sub.setTemperatures(temps[subset])
    bds = svm.brownianDynamics()
    bds.setModel(sub)
    bds.setDeltaT(PARAMS["dt"])
    singles, sbd = [], []
    for k, r in enumerate(subset):
        m = _single_from_state(svm, starts[k], float(sub.radii[k]), float(p0s[r]))
        d = svm.brownianDynamics()
        d.setModel(m)
        d.setDeltaT(PARAMS["dt"])
        d.setT(float(temps[r]))
        singles.append(m)
        sbd.append(d)
    nrng = np.random.default_rng(BATCH_SEED + 11)
    checkpoints = sorted({c for c in (10, 100, 1000, args.compare_steps) if c <= args.compare_steps})
    traj = {}
    for step in range(1, args.compare_steps + 1):
        xi = nrng.standard_normal((sub.nVertices, 3))
        bds.injectNoise(xi)
        bds.integrateEquationOfMotion()
        for k in range(len(subset)):
            sbd[k].injectNoise(xi[sub.vertexSlice(k)])
            sbd[k].integrateEquationOfMotion()
        if step in checkpoints:
            sub.computeGeometry()
            em = sub.replicaEnergies()
            rel = []
            for k, m in enumerate(singles):
                m.computeGeometry()
                e64 = m.computeEnergy()
                rel.append(abs(em[k] - e64) / abs(e64))
            rel = np.array(rel)
            traj[str(step)] = {"median": float(np.median(rel)), "q90": float(np.quantile(rel, 0.9)),
                               "max": float(rel.max())}
    sub_status = [sub.deviceStatus()] + [m.deviceStatus() for m in singles]
    for m in singles:
        m.close()
    sub.close()
    same = np.array(same)
    out = {"mode": "batch", "workload": f"{n_rep} replicas, N log-uniform [100, 5000] cells (total {int(sizes.sum())} "
                                        f"cells, {nv_all} vertices), P0 U[3.6, 3.95], T logU[1e-4, 1e-1], dt 0.01, "
                                        f"mixed form, T1 on, {steps_done} steps",
           "steps": steps_done, "ms_per_step": ms, "value": nv_all / (ms * 1e-3), "unit": UNIT,
           "t1_flips_per_step": t1["flips"] / (chunk * n_chunks), "device_status": status,
           "fp64_subset": {"replicas": [int(r) for r in subset],
                           "same_state_energy_rel_error": {"median": float(np.median(same)),
                                                           "q90": float(np.quantile(same, 0.9)),
                                                           "max": float(same.max())},
                           "trajectory_energy_rel_error_by_step": traj,
                           "trajectory": f"subset batch (mixed) vs FP64 singles from the prepared states, the same "
                                         f"injected normals, {args.compare_steps} steps",
                           "device_status": sub_status}}
    print(json.dumps(out), flush=True)


def mode_profile(args):
    """A small, untimed run for profilers (e.g. ncu -k regex:k_force_bd): a model of args.cells
    cells from the seeded recipe, args.stab stabilisation steps (T = 0, P0 = 1) one by one,
    args.equil graph-replayed steps at the run parameters, then args.steps Brownian steps at
    T = 0.01, P0 = 3.8 one launch per kernel per step (no graph), and the energy per cell.  --mixed
    runs those steps in the mixed form; --replicas R runs a batch of R replicas instead
    (stabilisation, then args.steps steps at per-replica P0 and T); --fire K adds K FIRE iterations
    (the reference's default parameters, force tolerance 1e-12 so that all K run, in the force form
    --fire-form, timed per iteration with the host synchronised on both sides); --neighbors K,
    K neighbour-list computations (range 1, radius R + 2.5); --active K, K self-propelled then K
    Vicsek steps; --dynamics K, K MSD + overlap evaluations (each printing its mean time)."""
    import numpy as np
    import curvedspacevertexmodel_gb300 as svm
    t0 = time.time()
    if args.replicas:
        rng = np.random.default_rng(SEED)
        sizes = np.exp(rng.uniform(np.log(100), np.log(5000), args.replicas)).astype(int)
        b = svm.sphericalVertexModelBatch(sizes, SEED + np.arange(args.replicas), p0=1.0)
        b.setT1Threshold(PARAMS["t1"])
        bd = svm.brownianDynamics()
        bd.setModel(b)
        b.setTemperatures(np.zeros(args.replicas))
        for _ in range(args.stab):
            bd.integrateEquationOfMotion()
        b.setPreferredParameters(1.0, rng.uniform(3.6, 3.95, args.replicas))
        b.setTemperatures(np.exp(rng.uniform(np.log(1e-4), np.log(1e-1), args.replicas)))
        for _ in range(args.steps):
            bd.integrateEquationOfMotion()
        b.computeGeometry()
        e = b.replicaEnergies() / sizes
        print(json.dumps({"mode": "profile", "replicas": args.replicas, "cells": b.nCells, "vertices": b.nVertices,
                          "median_energy_per_cell": float(np.median(e)), "status": b.deviceStatus(),
                          "wall_s": time.time() - t0}), flush=True)
        return
    noise = svm.noiseSource()
    noise.setReproducibleSeed(SEED)
    m = svm.sphericalVertexModel(args.cells, noise, 1.0, 3.8)
    m.setT1Threshold(PARAMS["t1"])
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(SEED + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    for _ in range(args.stab):
        bd.integrateEquationOfMotion()
    bd.setT(PARAMS["T"])
    m.setPreferredParameters(1.0, 3.8)
    if args.equil:
        bd.run(args.equil)
    if args.mixed:
        m.precision = "mixed"
    for _ in range(args.steps):
        bd.integrateEquationOfMotion()
    out = {"mode": "profile", "cells": args.cells, "vertices": m.nVertices}
    if args.fire:
        m.precision = args.fire_form
        fire = svm.energyMinimizerFIRE(m)
        fire.setMaximumIterations(args.fire)
        fire.setForceCutoff(1e-12)
        m.synchronize()
        m.t1Stats()
        t1 = time.perf_counter()
        fire.minimize()
        m.synchronize()
        out["fire_ms_per_iteration"] = (time.perf_counter() - t1) / args.fire * 1e3
        out["fire_t1_per_iteration"] = {k: v / args.fire for k, v in m.t1Stats().items()}
        out["fire_form"] = args.fire_form
        m.precision = "fp64"
    if args.dynamics:
        dyn = svm.dynamicalFeatures(m)
        dyn._both(0.5)
        t1 = time.perf_counter()
        for _ in range(args.dynamics):
            msd, ov = dyn._both(0.5)
        out["dynamics_ms_per_evaluation"] = (time.perf_counter() - t1) / args.dynamics * 1e3
    if args.active:
        for name, upd in (("self_propelled", svm.sphericalSelfPropelledParticle()),
                          ("vicsek", svm.sphericalVectorialVicsek())):
            upd.setModel(m)
            upd.setDeltaT(0.01)
            upd.setV0(0.1)
            if name == "vicsek":
                upd.setEta(0.5)
            upd.integrateEquationOfMotion()
            m.deviceStatus()
            t1 = time.perf_counter()
            upd.run(args.active)
            out[name + "_ms_per_step"] = (time.perf_counter() - t1) / args.active * 1e3
    if args.neighbors:
        nl = svm.neighborList(1.0, m.radius + 2.5, args.sub_grid)
        nl.computeNeighborLists(m, fetch=False)  # sizes the lists
        t1 = time.perf_counter()
        for _ in range(args.neighbors):
            nl.computeNeighborLists(m, fetch=False)
        out["neighbor_list_ms"] = (time.perf_counter() - t1) / args.neighbors * 1e3
        out["neighbor_list_nmax"] = nl.Nmax
        nl.close()
    m.computeGeometry()
    out.update(energy_per_cell=m.computeEnergy() / args.cells, status=m.deviceStatus(), wall_s=time.time() - t0)
    print(json.dumps(out), flush=True)


def mode_fire_ablation(args):
    """Where FIRE's iterations go, and what any warm start could save (N = 20k, the fire_warm_start
    instances: P0 U[3.6, 3.8], start = stabilisation + 500 Brownian steps at T = 0.01, FIRE with the
    vector-form forces and T1 on).  (a) Plain FIRE driven phase by phase (velocity-Verlet step +
    fireStep, bit for bit minimize), recording the iteration at which max|F| first drops below each
    decade from 1e-1 to 1e-9 and the energy per cell above the final minimum at that point.  (b) FIRE
    to max|F| < 1e-9 from the final minimum itself after k Brownian steps at T: a start far closer
    to the minimum than any predictor's -- a lower bound on the iterations a warm start can leave."""
    import numpy as np
    import curvedspacevertexmodel_gb300 as svm
    from curvedspacevertexmodel_gb300 import _lib, warm_start as ws
    rng = np.random.default_rng(FIRE_SEED)
    rows = []
    levels = [1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9]
    for i, p0 in enumerate(rng.uniform(3.6, 3.8, args.fire_instances)):
        seed = FIRE_SEED + i
        m = ws.start_state(args.cells, float(p0), seed)
        start = m.saveState()
        fire = svm.energyMinimizerFIRE(m)
        fire.setFIREParameters(*ws.FIRE_PARAMS)
        fire.setCriterion(_lib.SVM_FIRE_MAX_FORCE)
        fire.setMaximumIterations(10 ** 9)
        m.computeForces()
        reached, e_at, it = {}, {}, 0
        while it < 100000:
            fire.integrateEquationOfMotion()
            fire.fireStep()
            it += 1
            if it % 10 == 0:
                f = fire.state()["max_force"]
                for level in levels:
                    if level not in reached and f < level:
                        reached[level], e_at[level] = it, ws.energy(m)
                if f < 1e-9:
                    break
        e_min = ws.energy(m)
        minimum = m.saveState()
        del fire
        near = {}
        for k, T in ((1, 0.01), (10, 0.01), (10, 0.001)):
            m.loadState(minimum)
            bd = svm.brownianDynamics()
            bd.setModel(m)
            bd.setT(T)
            bd.noise.setReproducibleSeed(seed + 77)
            m.precision = "fp64"
            bd.run(k)
            m.precision = "fp64_vector"
            e0 = ws.energy(m)
            its, secs, _ = ws.minimize(m, 1e-9)
            near[f"{k} steps at T={T}"] = {"iterations": its, "seconds": secs,
                                           "start_energy_per_cell_above_min": (e0 - e_min) / m.nCells,
                                           "end_energy_per_cell_minus_min": (ws.energy(m) - e_min) / m.nCells}
        m.loadState(start)
        e_start = ws.energy(m)
        its_p, secs_p, _ = ws.minimize(m, 1e-9)
        rows.append({"p0": float(p0), "seed": seed, "plain_iterations": its_p, "plain_seconds": secs_p,
                     "first_below": {str(level): reached.get(level) for level in levels},
                     "energy_per_cell_above_min_when_first_below": {str(level): (e_at[level] - e_min) / m.nCells
                                                                    for level in e_at},
                     "start_energy_per_cell_above_min": (e_start - e_min) / m.nCells,
                     "from_the_minimum_after_brownian_steps": near,
                     "best_near_start_over_plain_iterations": min(v["iterations"] for v in near.values()) / its_p})
        m.close()
    print(json.dumps({"mode": "fire-ablation", "workload": f"N={args.cells}, P0 U[3.6, 3.8], FIRE to max|F|<1e-9 "
                      "(vector-form forces, T1 on)", "rows": rows}), flush=True)


MODE_DEFAULTS = {  # cells, steps, stab, equil, replicas
    "headline": (N_CELLS, 200, 100, 200, 512),   # 200 steps: the area fallback (~1 step in 8 to 20) averages out
    "forms": (N_CELLS, 10000, 100, 200, 0),
    "large": (1_000_000, 5000, 100, 0, 0),
    "batch": (0, 10000, 100, 0, 512),
    "profile": (1_000_000, 1, 2, 0, 0),
    "fire-ablation": (20000, 0, 0, 0, 0),
}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default per mode)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--mode", choices=tuple(MODE_DEFAULTS), default="headline")
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--stab", type=int, default=None, help="untimed stabilisation steps (T=0, P0=1)")
    ap.add_argument("--equil", type=int, default=None, help="untimed equilibration steps before warm-up")
    ap.add_argument("--cpu-steps", type=int, default=25, help="steps of the one-core CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision form's secondary timing")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-replica secondary timing")
    ap.add_argument("--replicas", type=int, default=None)
    ap.add_argument("--no-fire", action="store_true", help="skip the FIRE warm-start comparison")
    ap.add_argument("--fire-instances", type=int, default=2)
    ap.add_argument("--ref-cores", type=int, default=0)
    ap.add_argument("--every", type=int, default=1000, help="forms: checkpoint interval")
    ap.add_argument("--compare-steps", type=int, default=2000, help="batch: steps of the FP64 trajectory comparison")
    ap.add_argument("--fire-cap", type=int, default=12000, help="large: FIRE iteration cap (0: no FIRE)")
    ap.add_argument("--ensemble-blocks", type=int, default=10,
                    help="large: blocks of 200 steps per form for the energy error bars (0: none)")
    ap.add_argument("--mixed", action="store_true", help="profile: the steps in the mixed form")
    ap.add_argument("--fire", type=int, default=0, help="profile: FIRE iterations after the steps")
    ap.add_argument("--fire-form", default="fp64_vector", choices=("fp64", "fp64_vector"),
                    help="profile: force form of the FIRE iterations")
    ap.add_argument("--neighbors", type=int, default=0, help="profile: neighbour-list computations")
    ap.add_argument("--sub-grid", type=int, default=1, help="profile: the neighbour list's subGridReduction")
    ap.add_argument("--active", type=int, default=0, help="profile: timed self-propelled and Vicsek steps")
    ap.add_argument("--dynamics", type=int, default=0, help="profile: timed MSD + overlap evaluations")
    args = ap.parse_args()
    cells, steps, stab, equil, replicas = MODE_DEFAULTS[args.mode]
    for k, v in (("cells", cells), ("steps", steps), ("stab", stab), ("equil", equil), ("replicas", replicas)):
        if getattr(args, k) is None:
            setattr(args, k, v)
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "headline":
        run_ours(args)
    else:
        {"forms": mode_forms, "large": mode_large, "batch": mode_batch, "profile": mode_profile,
         "fire-ablation": mode_fire_ablation}[args.mode](args)


if __name__ == "__main__":
    main()
