"""Large single sphere: N = 1,000,000 cells (1,999,996 vertices), the reference's initialisation
recipe (seeded Voronoi start; stabilisation at T = 0, P0 = 1 for 100 steps), then P0 = 3.75,
T = 0.005, dt = 0.01, T1 threshold 0.04, `steps` Brownian steps in the mixed-precision form
(captured graph), then a FIRE quench to max|F| < 1e-8 (FP64 vector-form forces, T1 on) from that
state, plain and with the learned warm start.  Prints one JSON line.

    python -m curvedspacevertexmodel_gb300.large_sphere --steps 5000
"""
from __future__ import annotations

import argparse
import json
import os
import time

from . import _lib
from .model import brownianDynamics, energyMinimizerFIRE, noiseSource, sphericalVertexModel
from . import warm_start as ws


def fire(m, tol, cap):
    f = energyMinimizerFIRE(m)
    p = list(ws.FIRE_PARAMS)
    p[7] = tol
    f.setFIREParameters(*p)
    f.setCriterion(_lib.SVM_FIRE_MAX_FORCE)
    f.setMaximumIterations(cap)
    m.synchronize()
    t0 = time.perf_counter()
    f.minimize()
    m.synchronize()
    dt = time.perf_counter() - t0
    st = f.state()
    del f
    return st["iterations"], dt, st["max_force"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--fire-cap", type=int, default=40000)
    ap.add_argument("--seed", type=int, default=1137)
    args = ap.parse_args()
    out = {"workload": f"N={args.cells}, P0=3.75, T=0.005, dt=0.01, T1 0.04, {args.steps} mixed-form Brownian steps, "
                       "then FIRE to max|F|<1e-8 (FP64 vector form, T1 on), plain vs learned warm start"}
    t0 = time.perf_counter()
    noise = noiseSource()
    noise.setReproducibleSeed(args.seed)
    m = sphericalVertexModel(args.cells, noise)
    out["setup_s"] = time.perf_counter() - t0
    m.setT1Threshold(0.04)
    bd = brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(args.seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    bd.run(100)
    m.setPreferredParameters(1.0, 3.75)
    bd.setT(0.005)
    m.precision = "mixed"
    bd.run(10)
    m.t1Stats()
    m.synchronize()
    t0 = time.perf_counter()
    bd.run(args.steps)
    m.synchronize()
    dt = time.perf_counter() - t0
    t1 = m.t1Stats()
    out["brownian"] = {"ms_per_step": 1e3 * dt / args.steps, "vertex_steps_per_s": m.nVertices * args.steps / dt,
                       "t1_flips_per_step": t1["flips"] / args.steps, "device_status": m.deviceStatus(),
                       "area_fallback_taken_last_step": bool(m.areaCheck()[2])}
    m.computeGeometry()
    out["brownian"]["energy_per_cell"] = m.computeEnergy() / args.cells
    if args.fire_cap <= 0:
        print(json.dumps(out), flush=True)
        return
    m.precision = "fp64_vector"
    start = m.saveState()
    e0 = ws.energy(m)
    it, secs, fmax = fire(m, 1e-8, args.fire_cap)
    out["fire_plain"] = {"iterations": it, "seconds": secs, "max_force": fmax, "energy_per_cell": ws.energy(m) / args.cells,
                         "ms_per_iteration": 1e3 * secs / max(1, it), "device_status": m.deviceStatus()}
    m.loadState(start)
    net = ws.load(os.path.join(os.path.dirname(__file__), "data", "warm_start_n20k.npz"))
    m.synchronize()
    t0 = time.perf_counter()
    base = net.outputScale
    net.setOutputScale(0.25 * base)
    net.warmStart(m)
    e_w = ws.energy(m)
    fallback = None
    if e_w > e0:
        fallback = "warm start raised the energy"
        m.loadState(start)
    it_w, _, fmax_w = fire(m, 1e-8, args.fire_cap)
    m.synchronize()
    out["fire_warm"] = {"iterations": it_w, "seconds": time.perf_counter() - t0, "max_force": fmax_w,
                        "energy_start": e0, "energy_after_warm_start": e_w, "fallback": fallback,
                        "energy_per_cell": ws.energy(m) / args.cells, "device_status": m.deviceStatus()}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
