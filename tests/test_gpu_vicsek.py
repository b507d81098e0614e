"""Vicsek alignment of the vertex directors (sphericalVectorialVicsek, src/updaters/
sphericalVectorialVicsek.cpp:5-60) on the GPU against the CPU restatement, which is itself equal
bit for bit to the reference's updater (tests/test_oracle.py): the N=200 configuration with the
same uniform draws on both sides, and the in-kernel draws' limits."""
import numpy as np
import pytest

from gpu_helpers import gpu_model, load_gold, oracle_model, params, rel_err, same_rings, stabilised

pytestmark = pytest.mark.gpu
RTOL_STEP = 1e-12
RTOL_FREE = 1e-6    # free trajectories after 300 steps, as for the self-propelled updater
DT, MU, V0, ETA, TAU = 0.01, 1.0, 0.2, 0.5, 0.7


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def _vicsek(svm, m, eta=ETA, tau=TAU, dt=DT):
    vv = svm.sphericalVectorialVicsek()
    vv.setModel(m)
    vv.setDeltaT(dt)
    vv.setMu(MU)
    vv.setV0(V0)
    vv.setEta(eta)
    vv.setTau(tau)
    return vv


def test_vicsek_steps_match_oracle_from_the_same_state(svm, oracle_mod):
    """300 steps, the oracle restarted from the device's state (positions, connectivity,
    directors) before each one: flips, connectivity, positions and directors agree after every
    step to the last bits (the differences are the C library's and CUDA's acos, cos, sin)."""
    g = load_gold()
    p = params(g)
    gm = gpu_model(svm, g)
    om = oracle_model(oracle_mod, g)
    om.init_directors(oracle_mod.OracleNoise(31))
    gm.setDirectors(om.directors())
    vv = _vicsek(svm, gm)
    nz = oracle_mod.OracleNoise(78)
    nv, R = gm.nVertices, float(g["init_radius"])
    flips = 0
    for step in range(1, 301):
        rings, counts = gm.rings()
        om = oracle_mod.OracleModel(gm.returnPositions(), rings, counts, gm.vertexCellNeighbors(),
                                    gm.vertexNeighbors(), R)
        om.set_preferred(p["a0"], p["p0"])
        om.set_kr(p["kr"])
        om.set_t1_threshold(p["t1"])
        om.set_directors(gm.returnDirectors())
        uw = nz.uniforms(2 * nv, 0.0, 1.0)
        vv.injectNoise(uw)
        vv.integrateEquationOfMotion()
        om.vicsek_step_noise(uw, DT, MU, V0, ETA, TAU)
        fg, fo = gm.takeFlips(), om.flips()
        assert np.array_equal(fg, fo), step
        flips += len(fo)
        assert same_rings(gm, om), step
        assert np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors()), step
        assert rel_err(gm.returnPositions(), om.positions(), R) < RTOL_STEP, step
        assert rel_err(gm.returnDirectors(), om.directors()) < RTOL_STEP, step
    assert flips > 10
    assert gm.deviceStatus() == 0


def test_vicsek_trajectory_follows_oracle(svm, oracle_mod):
    """The same run free: the T1 flip list identical at every one of 300 steps and the
    trajectories apart by less than RTOL_FREE."""
    g = load_gold()
    gm = gpu_model(svm, g)
    om = oracle_model(oracle_mod, g)
    om.init_directors(oracle_mod.OracleNoise(31))
    gm.setDirectors(om.directors())
    vv = _vicsek(svm, gm)
    nz = oracle_mod.OracleNoise(78)
    nv, R = gm.nVertices, float(g["init_radius"])
    for step in range(1, 301):
        uw = nz.uniforms(2 * nv, 0.0, 1.0)
        vv.injectNoise(uw)
        vv.integrateEquationOfMotion()
        om.vicsek_step_noise(uw, DT, MU, V0, ETA, TAU)
        assert np.array_equal(gm.takeFlips(), om.flips()), step
    assert same_rings(gm, om)
    assert rel_err(gm.returnPositions(), om.positions(), R) < RTOL_FREE
    assert rel_err(gm.returnDirectors(), om.directors()) < RTOL_FREE


def test_vicsek_without_noise_is_the_neighbour_average(svm):
    """Eta = 0 and dt = tau: each new director is the tangent-projected, normalised average of
    the old directors of the vertex and its three neighbours (neighbours after the move's flips)."""
    m, _ = stabilised(svm, 20000, seed=3, stab=20, steps=10)
    vv = _vicsek(svm, m, eta=0.0, tau=DT)
    n0 = m.returnDirectors()
    vv.integrateEquationOfMotion()
    p = m.returnPositions()
    nb = m.vertexNeighbors()
    t = (n0 + n0[nb[:, 0]] + n0[nb[:, 1]] + n0[nb[:, 2]]) * 0.25
    t -= np.sum(t * p, axis=1, keepdims=True) / np.sum(p * p, axis=1, keepdims=True) * p
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    assert np.abs(m.returnDirectors() - t).max() < 1e-12
    assert m.deviceStatus() == 0


def test_vicsek_philox_noise_directions(svm):
    """Eta large and dt = tau: each new director is the in-kernel random tangent unit vector, whose
    angle in a tangent frame is uniform on the circle."""
    m, _ = stabilised(svm, 20000, seed=3, stab=20, steps=10)
    vv = _vicsek(svm, m, eta=1e7, tau=DT)
    vv.noise.setReproducibleSeed(9)
    vv.integrateEquationOfMotion()
    p = m.returnPositions()
    n1 = m.returnDirectors()
    ph = p / np.linalg.norm(p, axis=1, keepdims=True)
    assert np.abs(np.sum(n1 * ph, axis=1)).max() < 1e-12
    assert np.abs(np.linalg.norm(n1, axis=1) - 1).max() < 1e-12
    e1 = np.cross(ph, [0.0, 0.0, 1.0])
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(ph, e1)
    ang = np.arctan2(np.sum(n1 * e2, axis=1), np.sum(n1 * e1, axis=1))
    k = 4.0 / np.sqrt(ang.size)
    for f in (np.cos(ang), np.sin(ang), np.cos(2 * ang), np.sin(2 * ang)):
        assert abs(np.mean(f)) < k
    assert np.all(np.isfinite(n1)) and m.deviceStatus() == 0
