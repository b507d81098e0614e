"""The initial topology computed on the device (svm_topology_from_points_gpu) against the host
hull (svm_topology_from_points, itself checked against a qhull restatement and the reference's
construction): every array equal, for the seeded sphere recipe at sizes from a tetrahedron up,
and for clustered centres that need wider searches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


def _same(a, b):
    assert (a.nCells, a.nVertices, a.maxRing) == (b.nCells, b.nVertices, b.maxRing)
    assert np.array_equal(a.vertexPositions, b.vertexPositions)
    assert np.array_equal(a.vertexCells, b.vertexCells)
    assert np.array_equal(a.vertexNeighbors, b.vertexNeighbors)
    assert np.array_equal(a.ringCounts, b.ringCounts)
    assert np.array_equal(a.rings, b.rings)


@pytest.mark.parametrize("n,seed", [(4, 1), (5, 2), (12, 3), (80, 7), (200, 11), (1000, 13), (20000, 1137),
                                    (200000, 5)])
def test_device_hull_equals_host_hull(svm, n, seed):
    pts = svm.random_cell_centres(seed, n)
    _same(svm.Topology(pts, device=True), svm.Topology(pts))


def test_uneven_density(svm):
    """Two thirds of the centres on the northern hemisphere: the sparse south's stars need wider
    searches than the bins were sized for."""
    rng = np.random.default_rng(3)
    n = 6000
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    v[: 2 * n // 3, 2] = np.abs(v[: 2 * n // 3, 2])
    v[2 * n // 3:, 2] = -np.abs(v[2 * n // 3:, 2])
    pts = np.sqrt(n / (4 * np.pi)) * v
    _same(svm.Topology(pts, device=True), svm.Topology(pts))
