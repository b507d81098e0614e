"""Batches of replicas (svm_batch_*): every replica of a batch evolves exactly as the same sphere
run alone in the mixed-precision form (same noise, bit for bit, T1 flips included), per-replica
reductions agree with whole-batch ones, the autotuned launch gives the untuned trajectory, and
the batch's statistics agree with FP64 runs of the same replicas."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [120, 333, 57, 800, 210, 451]
SEEDS = [11, 12, 13, 14, 15, 16]
P0S = [3.6, 3.7, 3.75, 3.8, 3.9, 3.95]
TS = [1e-4, 1e-3, 3e-3, 1e-2, 3e-2, 1e-1]


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def make_batch(svm):
    b = svm.sphericalVertexModelBatch(SIZES, SEEDS, p0=P0S)
    b.setT1Threshold(0.04)
    b.setTemperatures(TS)
    return b


def make_single(svm, r):
    noise = svm.noiseSource()
    noise.setReproducibleSeed(SEEDS[r])
    m = svm.sphericalVertexModel(SIZES[r], noise, 1.0, P0S[r])
    m.setT1Threshold(0.04)
    m.precision = "mixed"
    return m


def test_batch_replicas_match_single_spheres_bitwise(svm):
    b = make_batch(svm)
    singles = [make_single(svm, r) for r in range(len(SIZES))]
    bdb = svm.brownianDynamics()
    bdb.setModel(b)
    bds = []
    for r, m in enumerate(singles):
        bd = svm.brownianDynamics()
        bd.setModel(m)
        bd.setT(TS[r])
        bds.append(bd)
    rng = np.random.default_rng(9)
    b.takeFlips()
    for m in singles:
        m.takeFlips()
    for step in range(40):
        xi = rng.standard_normal((b.nVertices, 3))
        bdb.injectNoise(xi)
        bdb.integrateEquationOfMotion()
        for r, (m, bd) in enumerate(zip(singles, bds)):
            bd.injectNoise(xi[b.vertexSlice(r)])
            bd.integrateEquationOfMotion()
    pos = b.returnPositions()
    vn = b.vertexNeighbors()
    vc = b.vertexCellNeighbors()
    rings, counts = b.rings()
    flips = b.takeFlips()
    total_flips = 0
    for r, m in enumerate(singles):
        vs, cs = b.vertexSlice(r), b.cellSlice(r)
        v0, c0 = vs.start, cs.start
        assert np.array_equal(pos[vs], m.returnPositions())
        assert np.array_equal(vn[vs] - v0, m.vertexNeighbors())
        assert np.array_equal(vc[vs] - c0, m.vertexCellNeighbors())
        rs, cnt = m.rings(b.ringCapacity)
        assert np.array_equal(counts[cs], cnt)
        mine = rings[cs]
        assert np.array_equal(np.where(mine >= 0, mine - v0, -1)[:, : rs.shape[1]], rs)
        fs = m.takeFlips()
        in_rep = (flips[:, 0] >= v0) & (flips[:, 0] < vs.stop)
        assert np.array_equal(flips[in_rep] - v0, fs)
        total_flips += len(fs)
    assert total_flips > 0
    assert b.deviceStatus() == 0


def test_batch_reductions(svm):
    b = make_batch(svm)
    bd = svm.brownianDynamics()
    bd.setModel(b)
    bd.run(50)
    b.computeGeometry()
    e = b.replicaEnergies()
    assert abs(e.sum() - b.computeEnergy()) < 1e-10 * b.computeEnergy()
    ap = b.areaPerimeter()
    pref_p0 = np.repeat(P0S, SIZES)
    for r in range(b.nReplicas):
        cs = b.cellSlice(r)
        er = np.sum((ap[cs, 0] - 1.0) ** 2 + (ap[cs, 1] - pref_p0[cs]) ** 2)
        assert abs(e[r] - er) < 1e-10 * er
    totals, excess, taken = b.replicaAreaCheck()
    R = b.radii
    assert np.all(np.abs(totals - 4 * np.pi * R * R) < 1e-9 * 4 * np.pi * R * R)
    assert not taken.any()


def test_autotuned_batch_gives_the_untuned_trajectory(svm):
    a, t = make_batch(svm), make_batch(svm)
    t.autotune(64, 256, 64, 1, 5)
    for m in (a, t):
        bd = svm.brownianDynamics()
        bd.setModel(m)
        bd.noise.setReproducibleSeed(5)
        bd.run(40)
        bd.run(40)
    bs = t.blockSizes()
    assert bs["samplingComplete"]
    assert all(bs[k] in (64, 128, 192, 256) for k in ("corners", "cells", "force"))
    assert np.array_equal(a.returnPositions(), t.returnPositions())
    assert np.array_equal(a.vertexNeighbors(), t.vertexNeighbors())


def test_batch_energies_track_fp64_singles(svm):
    """The batch (mixed form) and FP64 single-sphere runs of the same replicas, both prepared with
    the reference driver's stabilisation (T = 0, P0 = 1 for 100 steps) and then driven by the same
    injected noise for 300 steps at low temperature: per-replica energy per cell agrees to the
    separation that FP32 rounding builds up along the trajectory."""
    sizes, seeds, p0s = [1500, 2000, 2500, 3000], [21, 22, 23, 24], [3.6, 3.7, 3.75, 3.8]
    temps = [1e-4, 3e-4, 1e-4, 3e-4]
    b = svm.sphericalVertexModelBatch(sizes, seeds, p0=1.0)
    b.setT1Threshold(0.04)
    bdb = svm.brownianDynamics()
    bdb.setModel(b)
    b.setTemperatures([0.0] * 4)
    bdb.run(100)
    b.setPreferredParameters(1.0, p0s)
    b.setTemperatures(temps)
    singles, bds = [], []
    for r in range(4):
        noise = svm.noiseSource()
        noise.setReproducibleSeed(seeds[r])
        m = svm.sphericalVertexModel(sizes[r], noise, 1.0, 1.0)
        m.setT1Threshold(0.04)
        bd = svm.brownianDynamics()
        bd.setModel(m)
        bd.setT(0.0)
        bd.run(100)
        m.setPreferredParameters(1.0, p0s[r])
        bd.setT(temps[r])
        singles.append(m)
        bds.append(bd)
    rng = np.random.default_rng(4)
    for _ in range(300):
        xi = rng.standard_normal((b.nVertices, 3))
        bdb.injectNoise(xi)
        bdb.integrateEquationOfMotion()
        for r in range(4):
            bds[r].injectNoise(xi[b.vertexSlice(r)])
            bds[r].integrateEquationOfMotion()
    b.computeGeometry()
    eb = b.replicaEnergies() / np.array(sizes)
    for r in range(4):
        singles[r].computeGeometry()
        es = singles[r].computeEnergy() / sizes[r]
        print(f"replica {r}: energy/cell batch {eb[r]:.10g} fp64 {es:.10g} rel {abs(eb[r] - es) / es:.3e}")
        assert abs(eb[r] - es) < 5e-3 * es
    assert b.deviceStatus() == 0
