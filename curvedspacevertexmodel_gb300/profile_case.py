"""A small, self-contained run of the Brownian step for profilers (e.g. ncu -k regex:k_force_bd).

    python -m curvedspacevertexmodel_gb300.profile_case --cells 1000000 --stab 2 --steps 1

Builds a model of N cells from the seeded recipe, runs `stab` stabilisation steps (T = 0, P0 = 1,
as the reference driver does) and then `steps` Brownian steps at T = 0.01, P0 = 3.8, dt = 0.01
(T1 threshold 0.04), one launch per kernel per step (no graph), and prints the energy per cell.
With --mixed the `steps` steps run in the mixed-precision form (kernels k32_*).
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
    ap.add_argument("--seed", type=int, default=1137)
    ap.add_argument("--mixed", action="store_true", help="run the timed steps in the mixed-precision form")
    args = ap.parse_args()
    t0 = time.time()
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
    if args.mixed:
        m.precision = "mixed"
    for _ in range(args.steps):
        bd.integrateEquationOfMotion()
    m.computeGeometry()
    print(f"cells {args.cells} vertices {m.nVertices} energy/cell {m.computeEnergy() / args.cells:.6g} "
          f"status {m.deviceStatus()} wall {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main()
