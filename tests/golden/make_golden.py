"""Generates tests/golden/*.npz from the reference compiled from its own sources.

Run here (where the reference sources are present):
    make -C oracle/ref && python tests/golden/make_golden.py

The reference is built by oracle/ref/Makefile into oracle/_ref/libsvmref.so.  Fixture contents
(N = 200 cells, the Brownian configuration: A0 = 1, P0 = 3.8, Kr = 1, T = 0.01, mu = 1, dt = 0.01,
T1 threshold 0.04, cell centres from seed 1137, Brownian noise from seed 4242):
  * the initial topology, geometry, energy and forces;
  * positions, rings, vertex lists, areas/perimeters and energy after 1, 10, 100 and 1000 steps;
  * the T1 flips of the 1000 steps as (step, vertex1, vertex2), recorded by the oracle restatement
    while it is checked bit-for-bit against the reference at every step;
  * the reference cell list (cell size 1, radius R + 2.5) of the final vertex positions;
  * a FIRE quench (T1 off; dt 0.01, alpha0 0.1, dtMax 0.1, f_inc 1.1, f_dec 0.5, alphaDec 0.9,
    NMin 5) from the final Brownian state: positions after 100 iterations and after the full run.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

N, SEED, BD_SEED = 200, 1137, 4242
A0, P0, KR, T, MU, DT, T1 = 1.0, 3.8, 1.0, 0.01, 1.0, 0.01, 0.04
W = 16
CHECK = (1, 10, 100, 1000)
FIRE = dict(dt=0.01, alpha_start=0.1, dt_max=0.1, dt_inc=1.1, dt_dec=0.5, alpha_dec=0.9, n_min=5,
            force_cutoff=1e-13, alpha_min=0.0, max_iterations=4000)


def snapshot(m, prefix, out):
    # the reference keeps areaPerimeter from the start of the last step; recompute it for the
    # current positions (no effect on the trajectory: every step recomputes geometry first)
    m.compute_geometry()
    rings, counts = m.rings(W)
    out[prefix + "pos"] = m.positions()
    out[prefix + "rings"] = rings
    out[prefix + "counts"] = counts
    out[prefix + "vcells"] = m.vertex_cells()
    out[prefix + "vnbrs"] = m.vertex_neighbors()
    out[prefix + "ap"] = m.area_perimeter()
    out[prefix + "energy"] = np.array(m.energy())


def main():
    if not oracle.ref_available():
        raise SystemExit("build the reference first: make -C oracle/ref")
    oracle.build_oracle()
    ref = oracle.RefModel(N, SEED, A0, P0, KR, T1)
    out = {"params": np.array([N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1], dtype=np.float64)}
    snapshot(ref, "init_", out)
    out["init_radius"] = np.array(ref.radius)
    ref.compute_forces()
    out["init_forces"] = ref.forces()
    out["init_cellpos"] = ref.cell_positions()
    topo = ref.topology(W)
    orc = oracle.OracleModel(topo["pos"], topo["rings"], topo["counts"], topo["vcells"], topo["vnbrs"], topo["radius"])
    orc.set_preferred(A0, P0)
    orc.set_kr(KR)
    orc.set_t1_threshold(T1)
    ref.bd_setup(BD_SEED, T, DT, MU)
    noise = oracle.OracleNoise(BD_SEED)
    flips = []
    for step in range(1, CHECK[-1] + 1):
        ref.steps(1)
        orc.brownian_step(noise, T, DT, MU)
        for v1, v2 in orc.flips():
            flips.append((step, v1, v2))
        assert np.array_equal(ref.positions(), orc.positions()), step
        if step in CHECK:
            snapshot(ref, f"s{step}_", out)
            r1, c1 = ref.rings(W)
            r2, c2 = orc.rings(W)
            assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    out["flips"] = np.array(flips, dtype=np.int32).reshape(-1, 3)
    cl = ref.cell_list()
    nz = np.nonzero(cl["counts"])[0].astype(np.int32)
    out["cl_nside"] = np.array(cl["nside"])
    out["cl_nmax"] = np.array(cl["nmax"])
    out["cl_bins"] = nz
    out["cl_counts"] = cl["counts"][nz]
    out["cl_slots"] = cl["idx"][nz]
    # FIRE from the final Brownian state, T1 off
    ref.set_restricted(True)
    ref.fire_setup(**dict(FIRE, max_iterations=100))
    ref.steps(1)
    out["fire100_pos"] = ref.positions()
    out["fire100_force"] = np.array(oracle.ref_lib().ref_fire_force(ref.h))
    oracle.ref_lib().ref_fire_set_max_iterations(ref.h, FIRE["max_iterations"])
    ref.steps(1)
    out["fire_params"] = np.array([FIRE[k] for k in ("dt", "alpha_start", "dt_max", "dt_inc", "dt_dec", "alpha_dec",
                                                     "n_min", "force_cutoff", "alpha_min", "max_iterations")])
    out["fire_iterations"] = np.array(oracle.ref_lib().ref_fire_iterations(ref.h))
    out["fire_force"] = np.array(oracle.ref_lib().ref_fire_force(ref.h))
    out["fire_pos"] = ref.positions()
    ref.compute_geometry()
    out["fire_energy"] = np.array(ref.energy())
    np.savez_compressed(os.path.join(HERE, "brownian_n200.npz"), **out)
    print("flips", len(flips), "fire iterations", int(out["fire_iterations"]), "fire force", float(out["fire_force"]),
          "energy", float(out["s1000_energy"]), "->", float(out["fire_energy"]))


if __name__ == "__main__":
    main()
