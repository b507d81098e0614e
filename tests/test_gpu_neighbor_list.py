"""Neighbour lists on the device (svm_neighbor_list_*) against the oracle's restatement of
neighborList::computeCPU (src/utilities/neighborList.cpp:96-151): the width Nmax, every count,
index, minimum-image displacement and distance, bit for bit."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def _same(nl, ref):
    nm, npp, idx, vec, dist = ref
    assert nl.Nmax == nm
    assert np.array_equal(nl.neighborsPerParticle, npp)
    assert np.array_equal(nl.particleIndices, idx)
    assert np.array_equal(nl.neighborVectors, vec)
    assert np.array_equal(nl.neighborDistances, dist)


@pytest.mark.parametrize("sub_grid", [1, 2])
def test_model_vertices_match_oracle(svm, sub_grid):
    m = svm.sphericalVertexModel(6000, svm.noiseSource())
    R = m.radius
    nl = svm.neighborList(1.0, R + 2.5, sub_grid)
    nl.computeNeighborLists(m)
    ref = oracle.neighbor_list(m.returnPositions(), 1.0, R + 2.5, sub_grid)
    _same(nl, ref)
    assert nl.Nmax > 4 and nl.neighborsPerParticle.mean() > 3
    # a second call reuses the grown width
    nl.computeNeighborLists(m)
    _same(nl, ref)
    nl.close()


def test_device_points_in_a_periodic_box_match_oracle(svm):
    """Points filling the box, so that the minimum image crosses its faces."""
    import torch
    rng = np.random.default_rng(12)
    radius = 6.0
    pts = rng.uniform(-radius, radius * (1 - 1e-12), (5000, 3))
    pts[:40, 0] = radius * (1 - 1e-9)        # on the +x face ...
    pts[40:80, 0] = -radius                  # ... and on the -x face: neighbours through the boundary
    dev = torch.from_numpy(pts.copy()).cuda()
    for sub_grid, rng_ in ((1, 0.7), (2, 0.7), (3, 1.3)):
        nl = svm.neighborList(rng_, radius, sub_grid)
        nl.computeNeighborLists(dev)
        ref = oracle.neighbor_list(pts, rng_, radius, sub_grid)
        _same(nl, ref)
        wrapped = np.abs(nl.neighborVectors[:80, :, 0]).max()
        assert wrapped < rng_  # the displacement is the minimum image, not the raw difference
        nl.close()


def test_mixed_precision_model_is_listed_from_its_float_positions(svm):
    m = svm.sphericalVertexModel(3000, svm.noiseSource())
    m.precision = "mixed"
    R = m.radius
    nl = svm.neighborList(1.0, R + 2.5, 1)
    nl.computeNeighborLists(m)
    ref = oracle.neighbor_list(m.returnPositions().astype(np.float32).astype(np.float64), 1.0, R + 2.5, 1)
    _same(nl, ref)
    nl.close()


def test_crowded_bins_widen_the_cell_list(svm):
    """A bin holding more points than its slots: the cell list widens them and bins again, as the
    reference's grows its Nmax, and the lists still match."""
    import torch
    rng = np.random.default_rng(5)
    pts = rng.uniform(-3.0, 3.0, (600, 3))
    pts[:50] = 0.1 + rng.uniform(0.0, 0.05, (50, 3))   # 50 points in one bin
    nl = svm.neighborList(0.9, 3.0, 1, slotCapacity=4)
    nl.computeNeighborLists(torch.from_numpy(pts).cuda())
    ref = oracle.neighbor_list(pts, 0.9, 3.0, 1)
    _same(nl, ref)
    assert nl.Nmax >= 49
    nl.close()


def test_small_edge_cases(svm):
    """One point, a close pair, a pair across the periodic faces, a pair exactly at the range."""
    import torch
    small = [np.array([[0.5, -0.25, 1.0]]), np.array([[0.1, 0.2, 0.3], [0.15, 0.2, 0.3]]),
             np.array([[3.99, 0.0, 0.0], [-3.99, 0.0, 0.0]]), np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])]
    for pts in small:
        for sub in (1, 2):
            nl = svm.neighborList(0.5, 4.0, sub)
            nl.computeNeighborLists(torch.from_numpy(pts.copy()).cuda())
            _same(nl, oracle.neighbor_list(pts, 0.5, 4.0, sub))
            nl.close()
