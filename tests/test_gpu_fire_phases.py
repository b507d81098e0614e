"""The per-phase FIRE and velocity-Verlet entry points (svm_fire_step, svm_velocity_verlet_step,
svm_vv_half, svm_reduce_dots) through the C ABI: a loop of them reproduces svm_fire_minimize bit for
bit, and each matches the CPU restatement of the reference's fireStepCPU / integrateEOMCPU
(energyMinimizerFIRE.cpp:122-174, velocityVerlet.cpp:6-38)."""
import numpy as np
import pytest

from gpu_helpers import gpu_model, load_gold, oracle_model, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


@pytest.fixture(scope="module")
def gold():
    return load_gold()


def _fire(svm, m, fp, iters):
    f = svm.energyMinimizerFIRE(m)
    f.setFIREParameters(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), 1e-300, fp[8])
    f.setMaximumIterations(iters)
    return f


@pytest.mark.parametrize("restricted", [True, False])
def test_phase_loop_equals_minimize_bitwise(svm, gold, restricted):
    """minimize for K iterations against K rounds of (velocity-Verlet step at the minimizer's dt,
    fireStep): positions, velocities, forces, dt and alpha identical bit for bit (with T1 flips
    when motion is not restricted)."""
    fp = gold["fire_params"]
    K = 80
    a, b = gpu_model(svm, gold, "s1000_"), gpu_model(svm, gold, "s1000_")
    for m in (a, b):
        m.restrictedMotion = restricted
        m.setT1Threshold(0.08)   # flips happen while relaxing from the thermal state
    fa = _fire(svm, a, fp, K)
    fa.minimize()
    fb = _fire(svm, b, fp, K)
    b.computeForces()
    for _ in range(K):
        fb.integrateEquationOfMotion()
        fb.fireStep()
    assert fa.getCurrentIterations() == K
    assert np.array_equal(a.returnPositions(), b.returnPositions())
    assert np.array_equal(a.returnVelocities(), b.returnVelocities())
    assert np.array_equal(a.returnForces(), b.returnForces())
    sa, sb = fa.state(), fb.state()
    for k in ("dt", "alpha", "power", "n_since"):
        assert sa[k] == sb[k], k
    assert np.array_equal(a.vertexNeighbors(), b.vertexNeighbors())
    if not restricted:
        flips = len(b.takeFlips())
        assert len(a.takeFlips()) == flips and flips > 0
    assert a.deviceStatus() == 0 and b.deviceStatus() == 0


def test_velocity_verlet_matches_oracle(svm, gold, oracle_mod):
    """20 velocity-Verlet steps (dt 0.01, T1 on) from the golden thermal state with small random
    velocities: positions and velocities track the CPU restatement (acos is the only difference,
    and no noise drives the run); the flips are the same."""
    R = float(gold["init_radius"])
    rng = np.random.default_rng(3)
    v0 = rng.normal(0.0, 0.05, (396, 3))
    gm = gpu_model(svm, gold, "s1000_")
    om = oracle_model(oracle_mod, gold, "s1000_")
    gm.setVelocities(v0)
    om.set_velocities(v0)
    gm.computeForces()
    om.compute_forces()
    vv = svm.velocityVerlet()
    vv.setModel(gm)
    vv.setDeltaT(0.01)
    gm.takeFlips()
    om.flips()
    for step in range(20):
        vv.integrateEquationOfMotion()
        oracle_mod.vv_step(om, 0.01)
        assert np.array_equal(gm.takeFlips(), om.flips()), step
    assert rel_err(gm.returnPositions(), om.positions(), R) < 1e-11
    assert rel_err(gm.returnVelocities(), om.velocities()) < 1e-9
    assert gm.deviceStatus() == 0


def test_half_kick_and_dot_products(svm, gold):
    """svm_vv_half is v += dt/2 F exactly as the CPU rounds it; svm_reduce_dots returns sum F.v,
    sum F.F, sum v.v (to summation-order rounding) and max |F| (exactly)."""
    gm = gpu_model(svm, gold, "s100_")
    rng = np.random.default_rng(5)
    v0 = rng.normal(0.0, 0.1, (396, 3))
    gm.setVelocities(v0)
    gm.computeForces()
    f = gm.returnForces()
    vv = svm.velocityVerlet()
    vv.setModel(gm)
    vv.setDeltaT(0.02)
    vv.halfKick()
    v1 = gm.returnVelocities()
    assert np.array_equal(v1, v0 + (0.5 * 0.02) * f)
    d = svm.dotProducts(gm)
    fv = (f[:, 0] * v1[:, 0] + f[:, 1] * v1[:, 1]) + f[:, 2] * v1[:, 2]
    ff = (f[:, 0] * f[:, 0] + f[:, 1] * f[:, 1]) + f[:, 2] * f[:, 2]
    vvn = (v1[:, 0] * v1[:, 0] + v1[:, 1] * v1[:, 1]) + v1[:, 2] * v1[:, 2]
    scale = np.sum(np.abs(fv))
    assert abs(d["power"] - fv.sum()) < 1e-14 * scale
    assert abs(d["force_norm2"] - ff.sum()) < 1e-14 * ff.sum()
    assert abs(d["velocity_norm2"] - vvn.sum()) < 1e-14 * vvn.sum()
    assert d["max_force"] == np.sqrt(ff.max())


def test_fire_step_matches_oracle(svm, gold, oracle_mod):
    """One fireStep on the same forces and velocities: the velocity update and the dt/alpha
    control as fireStepCPU, for a positive and a negative power."""
    fp = gold["fire_params"]
    for sign in (1.0, -1.0):
        gm = gpu_model(svm, gold, "s100_")
        om = oracle_model(oracle_mod, gold, "s100_")
        gm.computeForces()
        om.compute_forces()
        v0 = sign * 0.3 * om.forces() + np.random.default_rng(1).normal(0, 1e-3, (396, 3))
        gm.setVelocities(v0)
        om.set_velocities(v0)
        f = _fire(svm, gm, fp, 10)
        of = oracle_mod.OracleFire(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), 1e-300, fp[8], 10)
        f.fireStep()
        of.fire_step(om)
        st, ost = f.state(), of.state()
        assert st["dt"] == ost["dt"] and st["alpha"] == ost["alpha"] and st["n_since"] == ost["n_since"]
        assert abs(st["power"] - ost["power"]) <= 1e-13 * abs(ost["power"])
        if sign > 0:
            assert rel_err(gm.returnVelocities(), om.velocities()) < 1e-13
        else:  # P <= 0: both set every velocity to zero
            assert not np.any(gm.returnVelocities()) and not np.any(om.velocities())


def test_per_phase_entry_points_reject_the_mixed_form(svm, gold):
    import ctypes as C
    from curvedspacevertexmodel_gb300 import _lib
    gm = gpu_model(svm, gold)
    gm.precision = "mixed"
    lib = _lib.lib()
    assert lib.svm_velocity_verlet_step(gm.handle, C.c_double(0.01), 1) == _lib.SVM_ERR_ARG
    assert lib.svm_vv_half(gm.handle, C.c_double(0.01)) == _lib.SVM_ERR_ARG
    assert lib.svm_reduce_dots(gm.handle, np.empty(4)) == _lib.SVM_ERR_ARG
