"""Generates tests/golden/next_rows.npz from the reference compiled from its own sources, for the
rows built beside the step: neighbour lists, the self-propelled and Vicsek updaters, the dynamical
observables and the save schedule.

Run here (where the reference sources are present):
    make -C oracle/ref && python tests/golden/make_golden_next.py

Fixture contents (every array made by the reference's own classes in oracle/_ref):
  * nl_box_*: neighborList(0.7, 3.0, 2) over 300 seeded points filling the periodic box
    (minimum images across its faces): Nmax, counts, indices, displacements, distances;
  * nl_model_*: neighborList(1.0, R + 2.5, 1) over the vertices of the N = 60 sphere (seed 7);
  * active{0,1}_*: the N = 120 sphere (seed 7; A0 1, P0 3.8, Kr 1, T1 threshold 0.04), its
    topology (initial positions pos0) and its directors (drawn by the reference from a
    random_device-seeded source, so they change when the file is regenerated), then 100 steps of
    sphericalSelfPropelledParticle (0) or sphericalVectorialVicsek (1) with the updater's noise
    seeded 55 (dt 0.01, mu 1, v0 0.3, Eta 0.5, tau 0.7): final positions and directors;
  * dyn_*: dynamicalFeatures' MSD and overlap of two seeded sphere configurations for three
    (fraction, cutoff) pairs;
  * lsi_*: logSpacedIntegers(37, 0.05), its first 150 save steps.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

ACTIVE = dict(dt=0.01, mu=1.0, v0=0.3, eta=0.5, tau=0.7)


def main():
    assert oracle.ref_available(), "build oracle/_ref first (make -C oracle/ref)"
    out = {}
    rng = np.random.default_rng(20)
    box = rng.uniform(-3.0, 3.0 * (1 - 1e-12), (300, 3))
    box[:12, 0] = 3.0 * (1 - 1e-9)
    box[12:24, 0] = -3.0
    nm, npp, idx, vec, dist = oracle.neighbor_list(box, 0.7, 3.0, 2, reference=True)
    out.update(nl_box_pts=box, nl_box_nmax=nm, nl_box_npp=npp, nl_box_idx=idx, nl_box_vec=vec, nl_box_dist=dist)
    small = oracle.RefModel(60, 7)
    pts = small.positions()
    nm, npp, idx, vec, dist = oracle.neighbor_list(pts, 1.0, small.radius + 2.5, 1, reference=True)
    out.update(nl_model_pts=pts, nl_model_radius=small.radius + 2.5, nl_model_nmax=nm, nl_model_npp=npp,
               nl_model_idx=idx, nl_model_vec=vec, nl_model_dist=dist)
    for kind in (0, 1):
        ref = oracle.RefModel(120, 7, 1.0, 3.8, 1.0, 0.04)
        topo = ref.topology()
        for k in ("pos", "rings", "counts", "vcells", "vnbrs"):
            out[f"active{kind}_{k}0" if k == "pos" else f"active{kind}_{k}"] = topo[k]
        out[f"active{kind}_radius"] = topo["radius"]
        out[f"active{kind}_dir0"] = ref.directors()
        ref.active_setup(kind, 55, ACTIVE["dt"], ACTIVE["mu"], ACTIVE["v0"], ACTIVE["eta"], ACTIVE["tau"])
        ref.steps(100)
        out[f"active{kind}_pos"] = ref.positions()
        out[f"active{kind}_dir"] = ref.directors()
    R = 12.0
    a = rng.normal(size=(2000, 3))
    a *= R / np.linalg.norm(a, axis=1, keepdims=True)
    b = a + rng.normal(scale=0.4, size=a.shape)
    b *= R / np.linalg.norm(b, axis=1, keepdims=True)
    cases = np.array([[1.0, 0.5], [0.37, 0.2], [0.999, 2.0]])
    res = np.array([oracle.dynamics(a, b, R, f, c, reference=True) for f, c in cases])
    out.update(dyn_a=a, dyn_b=b, dyn_radius=R, dyn_cases=cases, dyn_out=res)
    out["lsi_steps"] = oracle.log_spaced(37, 0.05, 150, reference=True)
    path = os.path.join(HERE, "next_rows.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
