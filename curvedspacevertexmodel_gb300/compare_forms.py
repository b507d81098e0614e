"""The FP64 plain form against the FP32-bulk/FP64-area (mixed) form over many steps at N = 100k
cells (the reference's own recipe: seeded Voronoi start, stabilisation at T = 0 and P0 = 1 for 100
steps, then A0 = 1, P0 = 3.8, T = 0.01, dt = 0.01, T1 threshold 0.04).  Both forms start from the
same FP32-representable state and are driven by the same standard normals (host-generated,
injected each step), so they differ only by arithmetic.  Reported at checkpoints: energy per cell,
the relative energy difference, area and perimeter differences (cells matched by index), the
fraction of vertices whose neighbours agree, the T1 flips of the last interval in both forms and
how many of them coincide (the same edge flipped in the same 200-step window), and each form's
step time (host-synchronised, including the noise upload).

    python -m curvedspacevertexmodel_gb300.compare_forms --steps 10000 --every 1000
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .model import brownianDynamics, noiseSource, sphericalVertexModel


def prepared(n: int, seed: int):
    noise = noiseSource()
    noise.setReproducibleSeed(seed)
    m = sphericalVertexModel(n, noise)
    m.setT1Threshold(0.04)
    bd = brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    bd.run(100)
    bd.setT(0.01)
    m.setPreferredParameters(1.0, 3.8)
    bd.run(200)
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=100000)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--every", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=1137)
    args = ap.parse_args()
    a = prepared(args.cells, args.seed)
    st = a.saveState()
    st["pos"] = st["pos"].astype(np.float32).astype(np.float64)
    a.loadState(st)
    b = sphericalVertexModel(args.cells, topology=None, noise=_noise(args.seed), radius=a.radius)
    b.setT1Threshold(0.04)
    b.loadState(st)
    b.setPreferredParameters(1.0, 3.8)
    b.precision = "mixed"
    bda, bdb = brownianDynamics(), brownianDynamics()
    for bd, m in ((bda, a), (bdb, b)):
        bd.setModel(m)
        bd.setT(0.01)
    rng = np.random.default_rng(args.seed + 7)
    a.takeFlips()
    b.takeFlips()
    ta = tb = 0.0
    nfa = nfb = ncommon = 0
    for step in range(1, args.steps + 1):
        xi = rng.standard_normal((a.nVertices, 3))
        for bd, m in ((bda, a), (bdb, b)):
            bd.injectNoise(xi)
            m.synchronize()
            t0 = time.perf_counter()
            bd.integrateEquationOfMotion()
            m.synchronize()
            if m is a:
                ta += time.perf_counter() - t0
            else:
                tb += time.perf_counter() - t0
        if step % 200 == 0 or step % args.every == 0:  # the flip logs hold 65,536 flips
            fa, fb = a.takeFlips(), b.takeFlips()
            nfa += len(fa)
            nfb += len(fb)
            ncommon += len(set(map(tuple, fa)) & set(map(tuple, fb)))
        if step % args.every == 0:
            a.computeGeometry()
            b.computeGeometry()
            ea, eb = a.computeEnergy() / args.cells, b.computeEnergy() / args.cells
            apa, apb = a.areaPerimeter(), b.areaPerimeter()
            same_nb = np.mean(np.all(np.sort(a.vertexNeighbors(), 1) == np.sort(b.vertexNeighbors(), 1), 1))
            print(json.dumps({
                "step": step, "energy_per_cell_fp64": ea, "energy_per_cell_mixed": eb,
                "energy_rel_diff": abs(ea - eb) / ea,
                "area_abs_diff_median_max": [float(np.median(np.abs(apa[:, 0] - apb[:, 0]))),
                                             float(np.max(np.abs(apa[:, 0] - apb[:, 0])))],
                "perimeter_abs_diff_median_max": [float(np.median(np.abs(apa[:, 1] - apb[:, 1]))),
                                                  float(np.max(np.abs(apa[:, 1] - apb[:, 1])))],
                "same_neighbour_fraction": float(same_nb), "flips_fp64": nfa, "flips_mixed": nfb,
                "flips_common": ncommon, "ms_per_step_fp64": 1e3 * ta / step, "ms_per_step_mixed": 1e3 * tb / step,
                "status": [a.deviceStatus(), b.deviceStatus()]}), flush=True)
            nfa = nfb = ncommon = 0


def _noise(seed):
    n = noiseSource()
    n.setReproducibleSeed(seed)
    return n


if __name__ == "__main__":
    main()
