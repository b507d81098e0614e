"""A small, self-contained run of the Brownian step for profilers (e.g. ncu -k regex:k_force_bd).

    python -m curvedspacevertexmodel_gb300.profile_case --cells 1000000 --stab 2 --steps 1

Builds a model of N cells from the seeded recipe, runs `stab` stabilisation steps (T = 0, P0 = 1,
as the reference driver does), `equil` graph-replayed steps at the run parameters, and then
`steps` Brownian steps at T = 0.01, P0 = 3.8, dt = 0.01
(T1 threshold 0.04), one launch per kernel per step (no graph), and prints the energy per cell.
With --mixed the `steps` steps run in the mixed-precision form (kernels k32_*); with --replicas R
a batch of R replicas runs instead (stabilisation, then `steps` steps at per-replica P0 and T);
with --fire K the `steps` Brownian steps are followed by K FIRE iterations (energyMinimizerFIRE,
the reference's default parameters, force tolerance 1e-12 so that all K run); with --neighbors K
the vertices' neighbour list (range 1, radius R + 2.5, the model's own) is then computed K times
and the mean time of a computation (device lists, Nmax read back) is printed; with --active K,
K self-propelled steps (v0 0.1, tau 1, in-kernel draws) and then K Vicsek steps (Eta 0.5) are
timed, and with --dynamics K, K evaluations of the MSD and overlap against the starting cell
positions (each reading its two numbers back).
"""
from __future__ import annotations

import argparse
import time

import curvedspacevertexmodel_gb300 as svm


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--stab", type=int, default=2)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--equil", type=int, default=0,
                    help="graph-replayed steps at the run parameters (FP64) before the profiled steps")
    ap.add_argument("--seed", type=int, default=1137)
    ap.add_argument("--mixed", action="store_true", help="run the timed steps in the mixed-precision form")
    ap.add_argument("--replicas", type=int, default=0,
                    help="instead: a batch of this many replicas, N log-uniform in [100, 5000] (seeded), "
                         "P0 U[3.6, 3.95], T logU[1e-4, 1e-1]")
    ap.add_argument("--fire", type=int, default=0, help="FIRE iterations after the Brownian steps")
    ap.add_argument("--neighbors", type=int, default=0, help="neighbour-list computations after the steps")
    ap.add_argument("--sub-grid", type=int, default=1, help="the neighbour list's subGridReduction")
    ap.add_argument("--active", type=int, default=0, help="timed self-propelled and Vicsek steps")
    ap.add_argument("--dynamics", type=int, default=0, help="timed MSD + overlap evaluations")
    args = ap.parse_args()
    t0 = time.time()
    if args.replicas:
        import numpy as np
        rng = np.random.default_rng(args.seed)
        sizes = np.exp(rng.uniform(np.log(100), np.log(5000), args.replicas)).astype(int)
        b = svm.sphericalVertexModelBatch(sizes, args.seed + np.arange(args.replicas), p0=1.0)
        b.setT1Threshold(0.04)
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
        print(f"replicas {args.replicas} cells {b.nCells} vertices {b.nVertices} median energy/cell {np.median(e):.6g} "
              f"status {b.deviceStatus()} wall {time.time() - t0:.1f} s")
        return
    noise = svm.noiseSource()
    noise.setReproducibleSeed(args.seed)
    m = svm.sphericalVertexModel(args.cells, noise, 1.0, 3.8)
    m.setT1Threshold(0.04)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(args.seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    for _ in range(args.stab):
        bd.integrateEquationOfMotion()
    bd.setT(0.01)
    m.setPreferredParameters(1.0, 3.8)
    if args.equil:
        bd.run(args.equil)
    if args.mixed:
        m.precision = "mixed"
    for _ in range(args.steps):
        bd.integrateEquationOfMotion()
    if args.fire:
        fire = svm.energyMinimizerFIRE(m)
        fire.setMaximumIterations(args.fire)
        fire.setForceCutoff(1e-12)
        fire.minimize()
    if args.dynamics:
        dyn = svm.dynamicalFeatures(m)
        dyn._both(0.5)
        t1 = time.perf_counter()
        for _ in range(args.dynamics):
            msd, ov = dyn._both(0.5)
        dt = (time.perf_counter() - t1) / args.dynamics
        print(f"dynamics: {m.nCells} cells, msd {msd:.4g} overlap {ov:.4g}, {dt * 1e3:.3f} ms per evaluation")
    if args.active:
        for name, upd in (("self-propelled", svm.sphericalSelfPropelledParticle()),
                          ("Vicsek", svm.sphericalVectorialVicsek())):
            upd.setModel(m)
            upd.setDeltaT(0.01)
            upd.setV0(0.1)
            if name == "Vicsek":
                upd.setEta(0.5)
            upd.integrateEquationOfMotion()
            m.deviceStatus()
            t1 = time.perf_counter()
            upd.run(args.active)
            st = m.deviceStatus()
            dt = (time.perf_counter() - t1) / args.active
            print(f"{name} step: {m.nVertices} vertices, {dt * 1e3:.3f} ms per step, status {st}")
    if args.neighbors:
        nl = svm.neighborList(1.0, m.radius + 2.5, args.sub_grid)
        nl.computeNeighborLists(m, fetch=False)  # sizes the lists
        t1 = time.perf_counter()
        for _ in range(args.neighbors):
            nl.computeNeighborLists(m, fetch=False)
        dt = (time.perf_counter() - t1) / args.neighbors
        print(f"neighbour list: {m.nVertices} points, Nmax {nl.Nmax}, {dt * 1e3:.3f} ms per computation")
        nl.close()
    m.computeGeometry()
    print(f"cells {args.cells} vertices {m.nVertices} energy/cell {m.computeEnergy() / args.cells:.6g} "
          f"status {m.deviceStatus()} wall {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main()
