"""Runs the GPU path and the CPU oracle side by side with the same (portable) arccosine and reports
how far apart they are.  Used by tests/test_gpu_portable_acos.py in a subprocess whose
SVM_LIBRARY is curvedspacevertexmodel_gb300/libsvm_pacos.so (the device library built with
-DSVM_PORTABLE_ACOS); the oracle is switched to the same function with set_portable_acos.

    SVM_LIBRARY=.../libsvm_pacos.so python tests/portable_acos_run.py n200|n20k|growth

Prints one JSON object: the number of steps and values compared and every difference found
(0 everywhere means bit for bit).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import curvedspacevertexmodel_gb300 as svm  # noqa: E402
import oracle  # noqa: E402
from gpu_helpers import gpu_model, load_gold, oracle_model, params, stabilised  # noqa: E402


def ndiff(a, b):
    """Elements whose bits differ."""
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.shape != b.shape:
        return -1
    return int(np.count_nonzero(a.view(np.uint64) != b.view(np.uint64)) if a.dtype == np.float64
               else np.count_nonzero(a != b))


def seq_energy(ap, pref, kr):
    """computeEnergy's sum in the CPU's cell order (sphericalVertexModel.cpp:150-160)."""
    e = 0.0
    for (a, p), (a0, p0) in zip(ap, pref):
        e += kr * (a - a0) * (a - a0) + (p - p0) * (p - p0)
    return e


def compare(gm, om, rep, kr, a0p0, full):
    rep["steps"] += 1
    rep["pos_bits_differ"] += ndiff(gm.returnPositions(), om.positions())
    rep["flips_differ"] += int(not np.array_equal(gm.takeFlips(), om.flips()))
    if full:
        rep["checks"] += 1
        rings_g, counts_g = gm.rings(32)
        rings_o, counts_o = om.rings(32)
        rep["topology_differ"] += int(not (np.array_equal(rings_g, rings_o) and np.array_equal(counts_g, counts_o)
                                           and np.array_equal(gm.vertexCellNeighbors(), om.vertex_cells())
                                           and np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors())))
        gm.computeGeometry()
        om.compute_geometry()
        ap_g, ap_o = gm.areaPerimeter(), om.area_perimeter()
        rep["area_perimeter_bits_differ"] += ndiff(ap_g, ap_o)
        pref = np.tile(a0p0, (ap_o.shape[0], 1))
        rep["energy_cpu_order_bits_differ"] += int(seq_energy(ap_g, pref, kr) != om.energy())
        e_dev = gm.computeEnergy()
        rep["energy_reduction_rel"] = max(rep["energy_reduction_rel"], abs(e_dev - om.energy()) / abs(om.energy()))


def run_n200(steps=1000):
    """The N = 200 Brownian configuration of the golden fixture, the reference's mt19937 normals
    injected into both sides; positions and flips compared after every step, everything else every
    50 steps and at the end."""
    g = load_gold()
    p = params(g)
    gm = gpu_model(svm, g)
    om = oracle_model(oracle, g)
    bd = svm.brownianDynamics()
    bd.setModel(gm)
    bd.setT(p["T"])
    bd.setDeltaT(p["dt"])
    bd.mu = p["mu"]
    noise = oracle.OracleNoise(p["bd_seed"])
    rep = dict(case="n200", steps=0, checks=0, pos_bits_differ=0, flips_differ=0, topology_differ=0,
               area_perimeter_bits_differ=0, energy_cpu_order_bits_differ=0, energy_reduction_rel=0.0, flips=0)
    for step in range(1, steps + 1):
        xi = noise.normals(3 * gm.nVertices)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, p["T"], p["dt"], p["mu"])
        rep["flips"] += len(om.flips(clear=False))
        compare(gm, om, rep, p["kr"], (p["a0"], p["p0"]), step % 50 == 0 or step in (1, 10, steps))
    rep["status"] = gm.deviceStatus()
    return rep


def run_n20k(steps=60):
    """N = 20k (the T1 pass spread over a cooperative grid) from the stabilised preparation: the
    oracle starts from the device's state and both run freely with the same injected normals."""
    m, _ = stabilised(svm, 20000, seed=8, stab=100, steps=100)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.setT(0.01)
    rings, counts = m.rings(16)
    om = oracle.OracleModel(m.returnPositions(), rings, counts, m.vertexCellNeighbors(), m.vertexNeighbors(), m.radius)
    om.set_preferred(1.0, 3.8)
    om.set_t1_threshold(0.04)
    m.takeFlips(1 << 20)
    noise = oracle.OracleNoise(99)
    rep = dict(case="n20k", steps=0, checks=0, pos_bits_differ=0, flips_differ=0, topology_differ=0,
               area_perimeter_bits_differ=0, energy_cpu_order_bits_differ=0, energy_reduction_rel=0.0, flips=0)
    for step in range(1, steps + 1):
        xi = noise.normals(3 * m.nVertices)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, 0.01, 0.01, 1.0)
        rep["flips"] += len(om.flips(clear=False))
        compare(m, om, rep, 1.0, (1.0, 3.8), step % 20 == 0)
    rep["status"] = m.deviceStatus()
    return rep


def run_growth(steps=700):
    """The N = 200 start at P0 = 4.2, T = 0.1, T1 threshold 0.2 with ring capacity 11 (its largest
    ring plus one) and no headroom: a ring fills the capacity, which grows before the next pass;
    compared with the restatement after every step."""
    g = load_gold()
    gm = gpu_model(svm, g, ring_capacity=11, ring_headroom=0)
    om = oracle_model(oracle, g)
    gm.setPreferredParameters(1.0, 4.2)
    gm.setT1Threshold(0.2)
    om.set_preferred(1.0, 4.2)
    om.set_t1_threshold(0.2)
    bd = svm.brownianDynamics()
    bd.setModel(gm)
    bd.setT(0.1)
    noise = oracle.OracleNoise(11)
    rep = dict(case="growth", steps=0, checks=0, pos_bits_differ=0, flips_differ=0, topology_differ=0,
               area_perimeter_bits_differ=0, energy_cpu_order_bits_differ=0, energy_reduction_rel=0.0, flips=0)
    for step in range(1, steps + 1):
        xi = noise.normals(3 * gm.nVertices)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, 0.1, 0.01, 1.0)
        rep["flips"] += len(om.flips(clear=False))
        compare(gm, om, rep, 1.0, (1.0, 4.2), step % 50 == 0)
    rep["status"] = gm.deviceStatus()
    rep["ring_info"] = gm.ringInfo()
    return rep


def main():
    if not os.environ.get("SVM_LIBRARY", "").endswith("libsvm_pacos.so"):
        raise SystemExit("run with SVM_LIBRARY pointing at libsvm_pacos.so")
    oracle.set_portable_acos(True)
    case = sys.argv[1] if len(sys.argv) > 1 else "n200"
    rep = {"n200": run_n200, "n20k": run_n20k, "growth": run_growth}[case]()
    print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    main()
