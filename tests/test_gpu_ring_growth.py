"""Ring capacity grows as the reference's growCellVerticesList (sphericalVertexModel.cpp:733-758)
widens its ring storage: no T1 flip is refused for want of storage, so a model started with a tight
capacity keeps following the reference flip for flip while its rings outgrow that capacity."""
import numpy as np
import pytest

from gpu_helpers import gpu_model, load_gold

pytestmark = pytest.mark.gpu

# A hot, fluid setting in which the golden N=200 start's largest ring (10) reaches 11 (the CPU
# restatement, from this noise stream, first gets there at step 427).
P0, T, THRESHOLD, NOISE_SEED, STEPS = 4.2, 0.1, 0.2, 11, 700


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def test_ring_driven_to_capacity_follows_the_oracle(svm, oracle_mod):
    """Capacity 11 (the start's largest ring plus one) and no headroom, so the capacity grows before
    the pass after one in which a ring filled it (the recorded maximum includes rings that were full
    only within a pass).  Every step starts the CPU restatement
    from the device's state and gives both the same normals: the flips of every step are equal (a
    refused flip would show here) and the device reports no overflow."""
    g = load_gold()
    gm = gpu_model(svm, g, ring_capacity=11, ring_headroom=0)
    assert gm.ringInfo()["capacity"] == 11
    gm.setPreferredParameters(1.0, P0)
    gm.setT1Threshold(THRESHOLD)
    bd = svm.brownianDynamics()
    bd.setModel(gm)
    bd.setT(T)
    noise = oracle_mod.OracleNoise(NOISE_SEED)
    R = float(g["init_radius"])
    grew_at, flips = None, 0
    for step in range(1, STEPS + 1):
        rings, counts = gm.rings(32)
        om = oracle_mod.OracleModel(gm.returnPositions(), rings, counts, gm.vertexCellNeighbors(),
                                    gm.vertexNeighbors(), R)
        om.set_preferred(1.0, P0)
        om.set_t1_threshold(THRESHOLD)
        xi = noise.normals(3 * gm.nVertices)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, T, 0.01, 1.0)
        fo = om.flips()
        assert np.array_equal(gm.takeFlips(), fo), step
        flips += len(fo)
        if grew_at is None and gm.ringInfo()["growths"]:
            grew_at = step
    info = gm.ringInfo()
    assert grew_at is not None and info["capacity"] > 11 and info["max_ring"] >= 11, info
    assert flips > 1000
    assert gm.deviceStatus() == 0


def test_graph_run_grows_like_the_step_loop(svm):
    """svm_brownian_run (captured pairs of steps, the capacity checked between replays) and the same
    steps one by one, from the golden N=200 start in the hot setting with capacity 12 and one slot
    of headroom: both grow their rings and end bit for bit equal, with no overflow."""
    g = load_gold()
    runs = []
    for graph in (True, False):
        m = gpu_model(svm, g, ring_capacity=12, ring_headroom=1)
        m.setPreferredParameters(1.0, P0)
        m.setT1Threshold(THRESHOLD)
        bd = svm.brownianDynamics()
        bd.setModel(m)
        bd.setT(T)
        bd.noise.setReproducibleSeed(5)
        if graph:
            bd.run(3000)
        else:
            for _ in range(3000):
                bd.integrateEquationOfMotion()
        runs.append((m.returnPositions(), m.vertexNeighbors(), m.rings(64), m.ringInfo(), m.deviceStatus()))
    (pa, na, ra, ia, sa), (pb, nb, rb, ib, sb) = runs
    assert sa == 0 and sb == 0, (sa, sb, ia, ib)
    assert ia["growths"] >= 1 and ib["growths"] >= 1, (ia, ib)
    assert np.array_equal(pa, pb) and np.array_equal(na, nb)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])


def test_host_buffer_steps_grow_like_the_step_loop(svm):
    """svm_brownian_step_io with page-locked buffers (a replayed graph per buffer role, the capacity
    checked before each replay) and the device-resident step loop, from the golden N=200 start in
    the hot setting with capacity 12 and one slot of headroom: both grow their rings and end bit for
    bit equal, with no overflow."""
    import ctypes as C
    import torch
    from curvedspacevertexmodel_gb300 import _lib
    g = load_gold()
    a = gpu_model(svm, g, ring_capacity=12, ring_headroom=1)
    b = gpu_model(svm, g, ring_capacity=12, ring_headroom=1)
    for m in (a, b):
        m.setPreferredParameters(1.0, P0)
        m.setT1Threshold(THRESHOLD)
    n = 3 * a.nVertices
    pos = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    out = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    pos[:] = a.returnPositions().reshape(-1)
    e_io = C.c_double()
    for _ in range(3000):
        _lib.call("svm_brownian_step_io", a.handle, T, 0.01, 1.0, 5, pos, out, C.byref(e_io))
        _lib.call("svm_brownian_step", b.handle, T, 0.01, 1.0, _lib.SVM_NOISE_PHILOX, None, 5)
        pos, out = out, pos
    ia, ib = a.ringInfo(), b.ringInfo()
    assert a.deviceStatus() == 0 and b.deviceStatus() == 0, (ia, ib)
    assert ia["growths"] >= 1 and ib["growths"] >= 1, (ia, ib)
    assert np.array_equal(pos.reshape(-1, 3), b.returnPositions())
    assert np.array_equal(a.vertexNeighbors(), b.vertexNeighbors())
    ra, rb = a.rings(64), b.rings(64)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])
