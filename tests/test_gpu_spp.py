"""Self-propelled vertices (sphericalSelfPropelledParticle, src/updaters/
sphericalSelfPropelledParticle.cpp:16-47) on the GPU against the CPU restatement: the N=200
configuration with the reference's uniform draws injected on both sides, and the in-kernel Philox
draws' distribution."""
import numpy as np
import pytest

from gpu_helpers import gpu_model, load_gold, oracle_model, params, rel_err, same_rings, stabilised

pytestmark = pytest.mark.gpu
RTOL_STEP = 1e-12
RTOL_SPP = 1e-6    # free trajectories after 300 steps (see the test)


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def _spp(svm, m):
    spp = svm.sphericalSelfPropelledParticle()
    spp.setModel(m)
    spp.setDeltaT(0.01)
    spp.setMu(1.0)
    spp.setV0(0.2)
    spp.setTau(1.0)
    return spp


def test_spp_steps_match_oracle_from_the_same_state(svm, oracle_mod):
    """v0 = 0.2, mu = 1, dt = 0.01, tau = 1 (Dr = 1), T1 threshold 0.04, N = 200: 300 steps, the
    oracle restarted from the device's state (positions, connectivity, directors) before each one:
    the ordered T1 flips, the connectivity, the positions and the directors agree after every
    step to the last bits (the only differences are the C library's and CUDA's acos, cos, sin)."""
    g = load_gold()
    p = params(g)
    gm = gpu_model(svm, g)
    om = oracle_model(oracle_mod, g)
    om.init_directors(oracle_mod.OracleNoise(31))
    gm.setDirectors(om.directors())
    assert np.array_equal(gm.returnDirectors(), om.directors())
    spp = _spp(svm, gm)
    nz = oracle_mod.OracleNoise(77)
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
        r = nz.uniforms(nv, -0.5, 0.5)
        spp.injectNoise(r)
        spp.integrateEquationOfMotion()
        om.spp_step_noise(r, 0.01, 1.0, 0.2, 1.0)
        fg, fo = gm.takeFlips(), om.flips()
        assert np.array_equal(fg, fo), step
        flips += len(fo)
        assert same_rings(gm, om), step
        assert np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors()), step
        assert rel_err(gm.returnPositions(), om.positions(), R) < RTOL_STEP, step
        assert rel_err(gm.returnDirectors(), om.directors()) < RTOL_STEP, step
    assert flips > 10
    assert gm.deviceStatus() == 0


def test_spp_trajectory_follows_oracle(svm, oracle_mod):
    """The same run free: the T1 flip list identical at every one of 300 steps and the trajectories
    apart by less than RTOL_SPP (measured: 3e-8 after 100 steps; the reference's gradients at
    collapsing edges amplify last-bit differences, as in the Brownian trajectories)."""
    g = load_gold()
    gm = gpu_model(svm, g)
    om = oracle_model(oracle_mod, g)
    om.init_directors(oracle_mod.OracleNoise(31))
    gm.setDirectors(om.directors())
    spp = _spp(svm, gm)
    nz = oracle_mod.OracleNoise(77)
    nv, R = gm.nVertices, float(g["init_radius"])
    for step in range(1, 301):
        r = nz.uniforms(nv, -0.5, 0.5)
        spp.injectNoise(r)
        spp.integrateEquationOfMotion()
        om.spp_step_noise(r, 0.01, 1.0, 0.2, 1.0)
        assert np.array_equal(gm.takeFlips(), om.flips()), step
    assert same_rings(gm, om)
    assert rel_err(gm.returnPositions(), om.positions(), R) < RTOL_SPP
    assert rel_err(gm.returnDirectors(), om.directors()) < RTOL_SPP


def test_spp_philox_rotation_angles(svm):
    """In-kernel draws: after one step, each director is the projected director rotated about its
    vertex's position vector p (length R) by theta, i.e. cos(theta) e1 + sin(theta) p x e1 with e1
    the projected unit director; theta is uniform on [-h, h], h = sqrt(2 dt tau) / 2."""
    m, _ = stabilised(svm, 20000, seed=3, stab=20, steps=10)
    spp = svm.sphericalSelfPropelledParticle()
    spp.setModel(m)
    spp.setDeltaT(0.01)
    spp.setTau(2.0)
    spp.setV0(0.1)
    spp.noise.setReproducibleSeed(5)
    n0 = m.returnDirectors()
    spp.integrateEquationOfMotion()
    p = m.returnPositions()
    n1 = m.returnDirectors()
    e1 = n0 - np.sum(n0 * p, axis=1, keepdims=True) / np.sum(p * p, axis=1, keepdims=True) * p
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(p, e1)
    R2 = np.sum(p * p, axis=1)
    theta = np.arctan2(np.sum(n1 * e2, axis=1) / R2, np.sum(n1 * e1, axis=1))
    h = 0.5 * np.sqrt(2 * 0.01 * 2.0)
    assert np.all(np.abs(theta) <= h * (1 + 1e-9))
    assert abs(np.mean(theta)) < 4 * h / np.sqrt(3 * theta.size)
    assert abs(np.var(theta) / (h * h / 3) - 1) < 0.03
    assert np.all(np.isfinite(n1)) and m.deviceStatus() == 0
