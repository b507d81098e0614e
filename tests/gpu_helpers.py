"""Shared helpers of the GPU tests: models built from the golden fixtures and the oracle."""
import numpy as np

GOLD = "tests/golden/brownian_n200.npz"

# How far the reference's own N = 200 trajectory moves when only the last bits of its arccosine
# change.  The CPU restatement (bit-exact with the reference build, which uses glibc's acos) is run
# with twelve other faithful arccosines -- the portable one (csrc/svm_acos.h, within 1.35 ulp of the
# exact value) and eleven seeded variants of glibc's with one result in four moved by one ulp
# (oracle.set_acos_mode) -- and compared with the golden fixture after 10, 100 and 1000 steps; the
# largest of the twelve is kept: max position error over R, max per-cell relative area or perimeter
# error, relative energy error.  Re-measured by
# tests/test_oracle.py::test_reference_trajectory_spread_under_faithful_acos.
ACOS_SPREAD_VARIANTS = [(1, 0)] + [(2, seed) for seed in range(1, 12)]
ACOS_SPREAD = {
    10: dict(pos=2.092e-9, ap=4.080e-9, energy=3.406e-10),
    100: dict(pos=7.484e-9, ap=2.501e-8, energy=2.893e-9),
    1000: dict(pos=1.110e-9, ap=1.089e-9, energy=2.200e-10),
}


def traj_tol(step, quantity, margin=2.0):
    """Tolerance of a GPU-vs-reference trajectory comparison after `step` steps: 1e-12, or
    `margin` times the reference's own spread under faithful changes of acos (ACOS_SPREAD),
    whichever is larger."""
    d = ACOS_SPREAD.get(step)
    return max(1e-12, margin * d[quantity]) if d else 1e-12


def trajectory_deviation(positions, area_perimeter, energy, gold, step):
    """(max position error over R, max per-cell relative area/perimeter error, relative energy
    error) of a state against the golden fixture after `step` steps."""
    R = float(gold["init_radius"])
    gap = gold[f"s{step}_ap"]
    ge = float(gold[f"s{step}_energy"])
    return dict(pos=float(np.max(np.abs(positions - gold[f"s{step}_pos"])) / R),
                ap=float(np.max(np.abs(area_perimeter - gap) / np.abs(gap))),
                energy=abs(energy - ge) / ge)


def load_gold():
    return dict(np.load(GOLD))


def params(g):
    N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1 = g["params"]
    return dict(N=int(N), seed=int(SEED), bd_seed=int(BD_SEED), a0=A0, p0=P0, kr=KR, T=T, mu=MU, dt=DT, t1=T1)


def gpu_model(svm, g, prefix="init_", ring_capacity=16, ring_headroom=None):
    p = params(g)
    topo = svm.Topology.from_arrays(g[prefix + "pos"], g[prefix + "rings"], g[prefix + "counts"],
                                    g[prefix + "vcells"], g[prefix + "vnbrs"])
    m = svm.sphericalVertexModel(p["N"], topology=topo, a0=p["a0"], p0=p["p0"], radius=float(g["init_radius"]),
                                 ringCapacity=ring_capacity, ringHeadroom=ring_headroom)
    m.setScalarModelParameter(p["kr"])
    m.setT1Threshold(p["t1"])
    return m


def oracle_model(oracle, g, prefix="init_"):
    p = params(g)
    m = oracle.OracleModel(g[prefix + "pos"], g[prefix + "rings"], g[prefix + "counts"], g[prefix + "vcells"],
                           g[prefix + "vnbrs"], float(g["init_radius"]))
    m.set_preferred(p["a0"], p["p0"])
    m.set_kr(p["kr"])
    m.set_t1_threshold(p["t1"])
    return m


def rel_err(a, b, scale=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.max(np.abs(b)) if scale is None else scale
    return float(np.max(np.abs(a - b)) / s) if a.size else 0.0


def same_rings(gm, om, W=16):
    r1, c1 = gm.rings(W)
    r2, c2 = om.rings(W)
    return np.array_equal(c1, c2) and np.array_equal(r1, r2)


def stabilised(svm, n, seed=5, stab=100, steps=200):
    """The reference driver's preparation (sphericalVertex.cpp:104-125): T = 0 with P0 = 1, then
    Brownian steps at T = 0.01, P0 = 3.8 (a raw random-Voronoi start diverges at large N in the
    reference itself)."""
    noise = svm.noiseSource()
    noise.setReproducibleSeed(seed)
    m = svm.sphericalVertexModel(n, noise)
    m.setT1Threshold(0.04)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(seed + 1)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    bd.run(stab)
    bd.setT(0.01)
    m.setPreferredParameters(1.0, 3.8)
    bd.run(steps)
    return m, bd


def vector_forces(pos, rings, counts, ap, pref, cellpos, R, kr=1.0):
    """Host FP64 evaluation of the model force -dE/dv as vectors of position differences (the
    formulas of the mixed-precision kernels, written independently in numpy): per (vertex, cell)
    slot, -2 dP [g(v, last) + g(v, next)] - 2 Kr dA [t(v, last, c) + t(v, c, next)] with g the
    geodesic-length gradient and t the signed spherical-triangle-area gradient (Van Oosterom and
    Strackee's tan(E/2) = N / D, differentiated)."""
    pos = np.asarray(pos, dtype=np.float64)
    v_l, c_l, l_l, x_l = [], [], [], []
    for c in range(rings.shape[0]):
        ring = rings[c, : counts[c]]
        v_l.append(ring)
        l_l.append(np.roll(ring, 1))
        x_l.append(np.roll(ring, -1))
        c_l.append(np.full(len(ring), c))
    v, c, last, nxt = (np.concatenate(a) for a in (v_l, c_l, l_l, x_l))
    P = pos[v]
    r = np.linalg.norm(P, axis=1, keepdims=True)
    a = P / r

    def dot(x, y):
        return np.sum(x * y, axis=1, keepdims=True)

    def geo(d):
        t = d - dot(d, a) * a
        return -t / np.linalg.norm(t, axis=1, keepdims=True)

    def tri(beta, gamma):
        bg = np.cross(beta, gamma)
        bxc = np.cross(a, gamma) + np.cross(beta, a) + bg
        N = dot(a, bg)
        D = 4.0 - dot(beta, beta) - dot(gamma, gamma) + dot(beta, gamma)
        g = 2.0 * (D * bxc - N * (beta + gamma)) / (N * N + D * D)
        return R * (g - dot(g, a) * a)

    dl, dx, dc = pos[last] - P, pos[nxt] - P, cellpos[c] - P
    dA = (ap[c, 0] - pref[c, 0])[:, None]
    dP = (ap[c, 1] - pref[c, 1])[:, None]
    fs = -2.0 * dP * (geo(dl) + geo(dx)) - 2.0 * kr * dA * (tri(dl / r, dc / r) + tri(dc / r, dx / r))
    f = np.zeros_like(pos)
    np.add.at(f, v, fs)
    return f
