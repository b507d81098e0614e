"""Shared helpers of the GPU tests: models built from the golden fixtures and the oracle."""
import numpy as np

GOLD = "tests/golden/brownian_n200.npz"


def load_gold():
    return dict(np.load(GOLD))


def params(g):
    N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1 = g["params"]
    return dict(N=int(N), seed=int(SEED), bd_seed=int(BD_SEED), a0=A0, p0=P0, kr=KR, T=T, mu=MU, dt=DT, t1=T1)


def gpu_model(svm, g, prefix="init_", ring_capacity=16):
    p = params(g)
    topo = svm.Topology.from_arrays(g[prefix + "pos"], g[prefix + "rings"], g[prefix + "counts"],
                                    g[prefix + "vcells"], g[prefix + "vnbrs"])
    m = svm.sphericalVertexModel(p["N"], topology=topo, a0=p["a0"], p0=p["p0"], radius=float(g["init_radius"]),
                                 ringCapacity=ring_capacity)
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
