"""Learned warm start for FIRE: training pairs from plain FIRE runs, training on the GPU with the
library's own kernels, and the warm-vs-plain comparison.

Workload (FIRE energy minimisation): N cells, P0 per instance, starting states = the reference
driver's stabilisation (100 steps at T = 0, P0 = 1; sphericalVertex.cpp:104-125) followed by 500
Brownian steps at T = 0.01 from the seeded Voronoi start; FIRE with dt0 = 0.01, alpha0 = 0.1,
dtMax = 0.1, f_inc = 1.1, f_dec = 0.5 (alphaDec 0.9, NMin 5, alphaMin 0: the reference's
setFIREParameters arguments, energyMinimizerFIRE.cpp:203-214) until max|F| < 1e-9, in FP64 with the
vector-form forces (the reference's closed forms floor max|F| near 1e-8 at N = 20k), T1 flips on
(with T1 off, collapsing edges leave cusps where max|F| cannot fall below ~0.1).

Warm start: the network moves every vertex by its predicted displacement (one fused kernel), and
FIRE runs from there to the same tolerance.  Plain FIRE from the unperturbed start is the fallback,
taken when the warm start raises the energy or FIRE from it exceeds the iteration budget; the
reported warm time then includes the failed attempt.

    python -m curvedspacevertexmodel_gb300.warm_start train --pairs 32 --target-iterations 1000 --clip 0.99 \
        --out weights.npz
    python -m curvedspacevertexmodel_gb300.warm_start evaluate --weights weights.npz --instances 6
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib
from .model import brownianDynamics, energyMinimizerFIRE, noiseSource, sphericalVertexModel, warmStartNetwork

FIRE_PARAMS = (0.01, 0.1, 0.1, 1.1, 0.5, 0.9, 5, 1e-9, 0.0)  # dt, alpha0, dtMax, finc, fdec, alphaDec, NMin, fc, amin
T1_THRESHOLD = 0.04


def start_state(n: int, p0: float, seed: int, steps: int = 500) -> sphericalVertexModel:
    noise = noiseSource()
    noise.setReproducibleSeed(seed)
    m = sphericalVertexModel(n, noise)
    m.setT1Threshold(T1_THRESHOLD)
    bd = brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    bd.run(100)
    bd.setT(0.01)
    m.setPreferredParameters(1.0, p0)
    bd.run(steps)
    m.precision = "fp64_vector"
    return m


def minimize(m: sphericalVertexModel, tol: float = 1e-9, max_iterations: int = 100000):
    """FIRE to max|F| < tol: (iterations, wall seconds, final max|F|)."""
    fire = energyMinimizerFIRE(m)
    p = list(FIRE_PARAMS)
    p[7] = tol
    fire.setFIREParameters(*p)
    fire.setCriterion(_lib.SVM_FIRE_MAX_FORCE)
    fire.setMaximumIterations(max_iterations)
    m.synchronize()
    t0 = time.perf_counter()
    fire.minimize()
    m.synchronize()
    dt = time.perf_counter() - t0
    st = fire.state()
    del fire
    return st["iterations"], dt, st["max_force"]


def energy(m: sphericalVertexModel) -> float:
    m.computeGeometry()
    return m.computeEnergy()


def align(p0: np.ndarray, p1: np.ndarray) -> np.ndarray:
    """p1 rotated about the sphere's centre to best match p0 (Kabsch, least squares): removes the
    rigid rotation that costs no energy and that FIRE's inertia picks up, which no local feature
    can predict."""
    H = p1.T @ p0
    U, _, Vt = np.linalg.svd(H)
    D = np.diag([1.0, 1.0, np.sign(np.linalg.det(Vt.T @ U.T))])
    Rm = Vt.T @ D @ U.T
    return p1 @ Rm.T


def training_pairs(n: int, p0s, seeds, tol: float = 1e-7, iterations: int = 0):
    """Features of each start state and, as targets, each vertex's displacement to its FIRE minimum
    (rigidly rotated back onto the start) in its start frame; vertices whose neighbours changed
    during the minimisation (T1) are left out.  Returns CUDA tensors X [S, 24], T [S, 2]."""
    import torch
    xs, ts = [], []
    for p0, seed in zip(p0s, seeds):
        m = start_state(n, float(p0), int(seed))
        m.computeForces()
        X, F = warmStartNetwork.features(m, frames=True)
        pos0, nb0 = m.returnPositions(), np.sort(m.vertexNeighbors(), axis=1)
        if iterations:
            minimize(m, tol, max_iterations=iterations)  # the first phase of the relaxation only
        else:
            minimize(m, tol)
        pos1, nb1 = m.returnPositions(), np.sort(m.vertexNeighbors(), axis=1)
        keep = np.all(nb0 == nb1, axis=1)
        fr = F.cpu().numpy()
        d = align(pos0, pos1) - pos0
        T = np.stack([np.sum(d * fr[:, :3], 1), np.sum(d * fr[:, 3:], 1)], 1)
        idx = torch.from_numpy(np.nonzero(keep)[0]).cuda()
        xs.append(X.index_select(0, idx))
        ts.append(torch.from_numpy(T[keep].astype(np.float32)).cuda())
        m.close()
    return torch.cat(xs), torch.cat(ts)


def train(X, T, epochs: int = 60, batch: int = 4096, lr: float = 1e-3, seed: int = 1):
    """A network trained on (X, T); the output scale is the targets' RMS."""
    scale = float(T.pow(2).mean().sqrt())
    net = warmStartNetwork(seed)
    net.setOutputScale(scale)
    losses = net.train(X, (T / scale).contiguous(), epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, scale, losses


def save(net: warmStartNetwork, path: str, meta: dict):
    np.savez(path, weights=net.weights(), scale=np.array(net.outputScale), meta=json.dumps(meta))


def load(path: str) -> warmStartNetwork:
    d = np.load(path)
    net = warmStartNetwork(1)
    net.setWeights(d["weights"])
    net.setOutputScale(float(d["scale"]))
    return net


def fallback_reason(e_start, e_after_warm_start, max_force_after=None, tolerance=1e-9):
    """Why plain FIRE from the unperturbed start must replace the warm-started run, or None: the
    warm start raised the energy, or FIRE from it missed the force tolerance within its iteration
    budget.  Written so that a NaN energy or force (a diverged warm start) takes the fallback."""
    if not (e_after_warm_start <= e_start):
        return "warm start raised the energy"
    if max_force_after is not None and not (max_force_after < tolerance):
        return "iteration budget exceeded"
    return None


def compare(net: warmStartNetwork, n: int, p0: float, seed: int, budget: float = 1.25, max_iterations: int = 100000,
            scales=(0.5, 0.25, 0.125)):
    """Plain FIRE and warm-started FIRE from the same start state (wall seconds and iterations).
    The warm start applies the predicted displacement at the step lengths `scales` and keeps the
    lowest energy; it falls back to plain FIRE when that still raises the energy or when FIRE from
    it needs more than `budget` x the plain run's iterations."""
    m = start_state(n, p0, seed)
    start = m.saveState()
    e0 = energy(m)
    it_p, t_p, f_p = minimize(m, max_iterations=max_iterations)
    e_plain = energy(m)
    m.loadState(start)
    m.synchronize()
    t0 = time.perf_counter()
    # the predicted displacement at a few step lengths; keep the lowest energy
    base = net.outputScale
    best = (None, None)
    for f in scales:
        if best[0] is not None:
            m.loadState(start)
        net.setOutputScale(base * f)
        net.warmStart(m)
        e = energy(m)
        if best[0] is None or e < best[0]:
            best = (e, f)
    net.setOutputScale(base)
    e_warm0, f_best = best
    if f_best != scales[-1]:
        m.loadState(start)
        net.setOutputScale(base * f_best)
        net.warmStart(m)
        net.setOutputScale(base)
    fallback = fallback_reason(e0, e_warm0)
    if fallback is None:
        cap = int(budget * it_p) if budget else max_iterations
        it_w, t_w, f_w = minimize(m, max_iterations=cap)
        fallback = fallback_reason(e0, e_warm0, f_w)
    if fallback:
        m.loadState(start)
        it_w, t_fb, f_w = minimize(m, max_iterations=max_iterations)
    m.synchronize()
    t_warm = time.perf_counter() - t0
    e_warm = energy(m)
    m.close()
    return dict(n=n, p0=p0, seed=seed, plain_s=t_p, plain_iterations=it_p, plain_max_force=f_p,
                warm_s=t_warm, warm_iterations=it_w, warm_max_force=f_w, fallback=fallback, warm_step_length=f_best,
                energy_start=e0, energy_after_warm_start=e_warm0, energy_per_cell_plain=e_plain / n,
                energy_per_cell_warm=e_warm / n, energy_per_cell_diff=abs(e_warm - e_plain) / n)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--cells", type=int, default=20000)
    tr.add_argument("--pairs", type=int, default=24)
    tr.add_argument("--epochs", type=int, default=60)
    tr.add_argument("--seed", type=int, default=3000)
    tr.add_argument("--target-iterations", type=int, default=0,
                    help="targets = displacement after this many FIRE iterations (0: to the minimum)")
    tr.add_argument("--clip", type=float, default=1.0, help="keep samples with |target| below this quantile")
    tr.add_argument("--out", required=True)
    ev = sub.add_parser("evaluate")
    ev.add_argument("--cells", type=int, default=20000)
    ev.add_argument("--instances", type=int, default=4)
    ev.add_argument("--seed", type=int, default=9000)
    ev.add_argument("--weights", required=True)
    args = ap.parse_args()
    rng = np.random.default_rng(args.seed)
    if args.cmd == "train":
        p0s = rng.uniform(3.6, 3.8, args.pairs)
        seeds = args.seed + np.arange(args.pairs)
        t0 = time.time()
        X, T = training_pairs(args.cells, p0s, seeds, iterations=args.target_iterations)
        t_pairs = time.time() - t0
        mag = T.norm(dim=1)
        q = [float(v) for v in mag.quantile(mag.new_tensor([0.5, 0.9, 0.99, 1.0])).cpu()] if mag.numel() < 16_000_000 \
            else []
        if args.clip < 1.0:
            keep = mag <= mag.quantile(args.clip)
            X, T = X[keep].contiguous(), T[keep].contiguous()
        net, scale, losses = train(X, T, epochs=args.epochs)
        meta = dict(cells=args.cells, pairs=args.pairs, p0s=list(map(float, p0s)), seeds=list(map(int, seeds)),
                    samples=int(X.shape[0]), epochs=args.epochs, pair_seconds=t_pairs, first_loss=losses[0],
                    target_quantiles_50_90_99_100=q, target_iterations=args.target_iterations, clip=args.clip,
                    last_loss=losses[-1], target_rms=scale)
        save(net, args.out, meta)
        print(json.dumps(meta))
    else:
        net = load(args.weights)
        p0s = rng.uniform(3.6, 3.8, args.instances)
        for i, p0 in enumerate(p0s):
            print(json.dumps(compare(net, args.cells, float(p0), args.seed + i)), flush=True)


if __name__ == "__main__":
    main()
