"""The C++ host layer (host/svm.hpp) through its example driver, a port of the reference's
Brownian driver: the same recipe through the Python classes gives the same energy, bit for bit
(both sit on the same C ABI)."""
import json
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def test_cpp_driver_matches_python_classes(svm):
    exe = os.path.join(os.path.dirname(svm.__file__), "sphericalVertex_gpu")
    assert os.path.exists(exe), "the build makes the C++ example"
    N, steps, T, p0, dt, seed = 200, 50, 0.01, 3.8, 0.01, 1137
    out = subprocess.run([exe, str(N), str(steps), str(T), str(p0), str(dt), str(seed)], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    cpp = json.loads(out.stdout.strip().splitlines()[-1])
    noise = svm.noiseSource()
    noise.setReproducibleSeed(seed)
    m = svm.sphericalVertexModel(N, noise, 1.0, p0)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(seed + 1)
    bd.setDeltaT(dt)
    bd.setT(0.0)
    m.setPreferredParameters(1.0, 1.0)
    for _ in range(steps):
        bd.integrateEquationOfMotion()
    bd.setT(T)
    m.setPreferredParameters(1.0, p0)
    for _ in range(steps):
        bd.integrateEquationOfMotion()
    m.computeGeometry()
    assert cpp["vertices"] == m.nVertices
    assert cpp["energy"] == m.computeEnergy()


def test_cpp_batch_matches_python_batch(svm):
    exe = os.path.join(os.path.dirname(svm.__file__), "sphericalVertex_gpu")
    N, steps, T, p0, dt, seed = 150, 40, 0.01, 3.7, 0.01, 21
    out = subprocess.run([exe, "batch", str(N), str(steps), str(T), str(p0), str(dt), str(seed)], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    cpp = json.loads(out.stdout.strip().splitlines()[-1])
    b = svm.sphericalVertexModelBatch([N, 2 * N, 3 * N], [seed, seed + 1, seed + 2], p0=p0)
    b.setT1Threshold(0.04)
    bd = svm.brownianDynamics()
    bd.setModel(b)
    bd.noise.setReproducibleSeed(seed + 7)
    bd.setDeltaT(dt)
    b.setTemperatures([T, 2 * T, 3 * T])
    for _ in range(steps):
        bd.integrateEquationOfMotion()
    b.computeGeometry()
    assert cpp["vertices"] == b.nVertices
    assert cpp["energies"] == list(b.replicaEnergies())


def test_cpp_vicsek_and_neighbour_list_match_python_classes(svm):
    """The Vicsek updater and the neighbour list through the C++ classes and through the Python
    classes: the same energy after 60 steps and the same lists, bit for bit."""
    import numpy as np
    exe = os.path.join(os.path.dirname(svm.__file__), "sphericalVertex_gpu")
    N, steps, seed = 300, 60, 41
    out = subprocess.run([exe, "active", str(N), str(steps), str(seed)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    cpp = json.loads(out.stdout.strip().splitlines()[-1])
    noise = svm.noiseSource()
    noise.setReproducibleSeed(seed)
    m = svm.sphericalVertexModel(N, noise, 1.0, 3.8)
    m.setT1Threshold(0.04)
    v = svm.sphericalVectorialVicsek()
    v.noise.setReproducibleSeed(seed + 3)
    v.setModel(m)
    v.setDeltaT(0.01)
    v.setV0(0.1)
    v.setEta(0.4)
    v.setTau(0.5)
    v.run(steps)
    m.computeGeometry()
    nl = svm.neighborList(1.0, m.radius + 2.5)
    nl.computeNeighborLists(m)
    assert cpp["vertices"] == m.nVertices
    assert cpp["energy"] == m.computeEnergy()
    assert cpp["Nmax"] == nl.Nmax
    assert cpp["pairs"] == int(nl.neighborsPerParticle.sum())
    assert cpp["index_sum"] == int(nl.particleIndices.astype(np.int64).sum())
    nl.close()


def test_cpp_fire_phases_match_python_classes(svm):
    """FIRE driven phase by phase through the C++ classes (velocityVerlet step + fireStep, then the
    dot products) and through the Python classes: the same energy and sums, bit for bit."""
    exe = os.path.join(os.path.dirname(svm.__file__), "sphericalVertex_gpu")
    N, iters, seed = 250, 60, 13
    out = subprocess.run([exe, "fire", str(N), str(iters), str(seed)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    cpp = json.loads(out.stdout.strip().splitlines()[-1])
    noise = svm.noiseSource()
    noise.setReproducibleSeed(seed)
    m = svm.sphericalVertexModel(N, noise, 1.0, 1.0)
    m.setT1Threshold(0.04)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.noise.setReproducibleSeed(seed + 1)
    for _ in range(50):
        bd.integrateEquationOfMotion()
    m.setPreferredParameters(1.0, 3.8)
    fire = svm.energyMinimizerFIRE(m)
    fire.setFIREParameters(0.01, 0.1, 0.1, 1.1, 0.5, 0.9, 5, 1e-300, 0.0)
    fire.setMaximumIterations(iters)
    m.computeForces()
    for _ in range(iters):
        fire.integrateEquationOfMotion()
        fire.fireStep()
    d = svm.dotProducts(m)
    m.computeGeometry()
    assert cpp["energy"] == m.computeEnergy()
    assert cpp["dots"] == [d["power"], d["force_norm2"], d["velocity_norm2"], d["max_force"]]
