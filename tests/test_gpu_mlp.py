"""The warm-start network's kernels against the CPU reference (oracle/mlp.py): forward pass,
hand-written backward pass (gradients), features of a model state, and that Adam training
through the device kernels learns a target the CPU reference defines."""
import numpy as np
import pytest

import mlp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def random_net(svm, seed):
    net = svm.warmStartNetwork(seed)
    w = np.random.default_rng(seed).normal(0, 0.25, net.parameterCount).astype(np.float32)
    net.setWeights(w)
    return net, w


def test_forward_matches_cpu_reference(svm, torch):
    net, w = random_net(svm, 3)
    X = np.random.default_rng(1).normal(0, 1, (3000, 24)).astype(np.float32)
    Y = net.predict(torch.from_numpy(X).cuda()).cpu().numpy()
    Yref, _ = mlp.forward(mlp.bf16(w), X.astype(np.float64))
    assert np.max(np.abs(Y - Yref)) < 1e-4 * max(1.0, np.max(np.abs(Yref)))


def test_gradient_matches_cpu_reference(svm, torch):
    net, w = random_net(svm, 4)
    rng = np.random.default_rng(2)
    X = rng.normal(0, 1, (2000, 24)).astype(np.float32)
    T = rng.normal(0, 1, (2000, 2)).astype(np.float32)
    loss, g = net.gradient(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    lref, gref = mlp.loss_and_grad(mlp.bf16(w), X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - lref) < 1e-5 * lref
    # FP32 accumulation; a ReLU pre-activation within rounding of zero may switch a sample's unit
    assert np.linalg.norm(g - gref) < 1e-4 * np.linalg.norm(gref)
    rel = np.abs(g - gref) / (np.abs(gref) + 1e-3 * np.max(np.abs(gref)))
    assert np.median(rel) < 1e-5


def test_features_match_cpu_reference(svm, torch):
    noise = svm.noiseSource()
    noise.setReproducibleSeed(8)
    m = svm.sphericalVertexModel(600, noise)
    m.setT1Threshold(0.04)
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.setT(0.01)
    bd.run(50)
    m.computeForces()
    X, F = svm.warmStartNetwork.features(m, frames=True)
    rings, counts = m.rings()
    Xref, e1, e2 = mlp.features(m.returnPositions(), m.vertexNeighbors(), m.vertexCellNeighbors(),
                                m.cellPositions(), m.areaPerimeter(), np.tile([1.0, 3.8], (600, 1)), counts,
                                m.returnForces())
    assert np.max(np.abs(X.cpu().numpy() - Xref)) < 1e-5
    assert np.max(np.abs(F.cpu().numpy() - np.concatenate([e1, e2], 1))) < 1e-12


def test_training_learns_a_teacher_network(svm, torch):
    rng = np.random.default_rng(5)
    teacher = rng.normal(0, 0.3, mlp.N_PARAMS)
    X = rng.normal(0, 1, (20000, 24))
    T, _ = mlp.forward(teacher, X)
    Xd = torch.from_numpy(X.astype(np.float32)).cuda()
    Td = torch.from_numpy(T.astype(np.float32)).cuda()
    net = svm.warmStartNetwork(11)
    losses = net.train(Xd, Td, epochs=60, batch=1024, lr=3e-3, seed=1)
    assert losses[-1] < 0.2 * losses[0]
    # the trained weights reproduce the device's own loss on the CPU reference
    lref, _ = mlp.loss_and_grad(mlp.bf16(net.weights()), X, T)
    l, _ = net.gradient(Xd, Td)
    assert abs(l - lref) < 1e-4 * lref


def test_zero_network_warm_start_keeps_the_state(svm):
    noise = svm.noiseSource()
    noise.setReproducibleSeed(9)
    m = svm.sphericalVertexModel(400, noise)
    net = svm.warmStartNetwork(1)
    net.setWeights(np.zeros(net.parameterCount, dtype=np.float32))
    p0 = m.returnPositions()
    net.warmStart(m)
    assert np.max(np.abs(m.returnPositions() - p0)) < 1e-12 * m.radius
