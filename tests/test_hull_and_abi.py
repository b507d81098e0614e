"""CPU tests of the host side: the spherical hull / initial topology (against scipy's qhull and
the Euler counts), the product's random cell centres (against the oracle restatement of the
reference recipe), and the C ABI (the library loads and exports every symbol include/svm.h
declares; no device work)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def svm(svm_lib):
    return svm_lib


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "svm.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(svm_\w+)\s*\(", text, re.M)))


def test_abi_exports_every_declared_symbol(svm):
    lib = ctypes.CDLL(svm.LIBPATH)
    names = declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi(svm):
    from curvedspacevertexmodel_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_cell_centres_match_reference_recipe(svm, oracle_mod):
    for seed, n in ((1137, 200), (5, 1000)):
        a = svm.random_cell_centres(seed, n)
        b = oracle_mod.OracleNoise(seed).cell_centres(n)
        assert np.array_equal(a, b)
        R = np.sqrt(n / (4 * svm.PI))
        assert np.allclose(np.linalg.norm(a, axis=1), R, rtol=1e-14)


@pytest.mark.parametrize("n,seed", [(12, 1), (200, 1137), (2000, 9), (20000, 3)])
def test_topology_against_qhull(svm, n, seed):
    spatial = pytest.importorskip("scipy.spatial")
    pts = svm.random_cell_centres(seed, n)
    topo = svm.Topology(pts)
    assert topo.nVertices == 2 * n - 4
    # the same triangle set as qhull
    hull = spatial.ConvexHull(pts)
    ours = set()
    cells = topo.vertexCells
    for f in range(topo.nVertices):
        ours.add(tuple(sorted(cells[f])))
    theirs = {tuple(sorted(s)) for s in hull.simplices}
    assert ours == theirs
    # Euler / incidence invariants
    counts = topo.ringCounts.astype(int)
    assert counts.sum() == 3 * topo.nVertices
    for c in range(0, n, max(1, n // 50)):
        ring = topo.rings[c, : counts[c]]
        for v in ring:
            assert c in cells[v]
    # vertices are the renormalised facet centroids
    R = np.linalg.norm(pts[0])
    cen = pts[cells].mean(axis=1)
    assert np.allclose(topo.vertexPositions, R * cen / np.linalg.norm(cen, axis=1, keepdims=True), rtol=1e-12)
    # vertex -> vertex slot k is the facet across the edge ending at corner k
    nbrs = topo.vertexNeighbors
    for f in range(0, topo.nVertices, max(1, topo.nVertices // 200)):
        for k in range(3):
            g = nbrs[f, k]
            shared = set(cells[f]) & set(cells[g])
            assert shared == {cells[f][(k + 2) % 3], cells[f][k]}


def test_rings_are_clockwise_from_outside(svm):
    pts = svm.random_cell_centres(1137, 200)
    topo = svm.Topology(pts)
    p = topo.vertexPositions
    for c in range(200):
        ring = topo.rings[c, : topo.ringCounts[c]]
        # signed area of the ring polygon about the outward normal at the cell centre
        nrm = pts[c] / np.linalg.norm(pts[c])
        s = 0.0
        for k in range(len(ring)):
            s += np.dot(np.cross(p[ring[k]], p[ring[(k + 1) % len(ring)]]), nrm)
        assert s < 0  # clockwise seen from outside


def test_topology_from_triangles_matches_hull(svm):
    spatial = pytest.importorskip("scipy.spatial")
    pts = svm.random_cell_centres(42, 500)
    hull = spatial.ConvexHull(pts)
    tri = hull.simplices.copy()
    # orient CCW seen from outside
    for t in tri:
        a, b, c = pts[t]
        if np.dot(np.cross(b - a, c - a), a) < 0:
            t[1], t[2] = t[2], t[1]
    t1 = svm.Topology(pts)
    t2 = svm.Topology(pts, triangles=tri)
    for name in ("vertexPositions", "rings", "ringCounts", "vertexCells", "vertexNeighbors"):
        assert np.array_equal(getattr(t1, name), getattr(t2, name)), name


def test_topology_matches_reference_hull_shim(svm, oracle_mod):
    if not oracle_mod.ref_available():
        pytest.skip("oracle/_ref not built")
    ref = oracle_mod.RefModel(200, 1137, 1.0, 3.8, 1.0, 0.04)
    t = ref.topology()
    topo = svm.Topology(svm.random_cell_centres(1137, 200))
    W = t["rings"].shape[1]
    assert np.array_equal(t["pos"], topo.vertexPositions)
    assert np.array_equal(t["rings"], topo.rings[:, :W])
    assert np.array_equal(t["vcells"], topo.vertexCells)
    assert np.array_equal(t["vnbrs"], topo.vertexNeighbors)


def test_oracle_topology_matches_product(svm, oracle_mod):
    """The reference leg builds its initial state without product code; it must agree."""
    pytest.importorskip("scipy.spatial")
    import topology as otopo
    pts = svm.random_cell_centres(1137, 300)
    t = otopo.topology(pts)
    topo = svm.Topology(pts)
    assert np.array_equal(t["pos"], topo.vertexPositions)
    assert np.array_equal(t["rings"], topo.rings)
    assert np.array_equal(t["counts"], topo.ringCounts)
    assert np.array_equal(t["vcells"], topo.vertexCells)
    assert np.array_equal(t["vnbrs"], topo.vertexNeighbors)


def test_abi_rejects_bad_arguments_without_a_device(svm):
    """Argument checks come before any device work: invalid sizes, null handles and pointers
    return SVM_ERR_ARG (no exception crosses the ABI, nothing touches a GPU)."""
    import ctypes as C
    L = svm.lib()
    h = C.c_void_p()
    ERR_ARG = 1
    assert L.svm_model_create(3, 2, 16, 1.0, None, C.byref(h)) == ERR_ARG          # N < 4
    assert L.svm_model_create(100, 197, 16, 1.0, None, C.byref(h)) == ERR_ARG      # Nv != 2N - 4
    assert L.svm_model_create(100, 196, 2, 1.0, None, C.byref(h)) == ERR_ARG       # ring capacity
    assert L.svm_model_create(100, 196, 16, -1.0, None, C.byref(h)) == ERR_ARG     # radius
    n = np.array([100, 3], dtype=np.int32)
    nv = np.array([196, 2], dtype=np.int32)
    r = np.array([1.0, 1.0])
    assert L.svm_batch_create(2, n, nv, 16, r, None, C.byref(h)) == ERR_ARG         # a replica with N < 4
    assert L.svm_batch_create(0, n, nv, 16, r, None, C.byref(h)) == ERR_ARG
    for fn in ("svm_model_compute_geometry", "svm_model_compute_forces", "svm_model_enforce_topology",
               "svm_model_destroy", "svm_fire_destroy", "svm_mlp_destroy", "svm_tuner_destroy"):
        assert getattr(L, fn)(None) == ERR_ARG, fn
    assert L.svm_model_set_precision(None, 1) == ERR_ARG
    assert L.svm_model_set_t1_blocks(None, 0) == ERR_ARG
    assert L.svm_brownian_step_io(None, 0.0, 0.01, 1.0, 1, None, None, None) == ERR_ARG
    assert L.svm_energy_noalloc(None, None, 1.0, 10, None, None) == ERR_ARG
    three = np.zeros(9)
    assert L.svm_topology_from_points_gpu(three, 3, None, C.byref(h)) == ERR_ARG  # N < 4
    for bad in ((0.0, 5.0, 1, 10, 16), (1.0, -1.0, 1, 10, 16), (1.0, 5.0, 0, 10, 16), (1.0, 5.0, 1, 0, 16)):
        rng_, rad, sub, npts, cap = bad
        assert L.svm_neighbor_list_create(C.c_double(rng_), C.c_double(rad), sub, npts, cap, None,
                                          C.byref(h)) == ERR_ARG, bad
    for fn in ("svm_neighbor_list_destroy",):
        assert getattr(L, fn)(None) == ERR_ARG, fn
    assert L.svm_neighbor_list_compute(None, None, 10) == ERR_ARG
    assert L.svm_neighbor_list_compute_model(None, None) == ERR_ARG
    assert L.svm_vicsek_step(None, C.c_double(0.01), C.c_double(1.0), C.c_double(0.1), C.c_double(0.5),
                             C.c_double(1.0), 1, None, C.c_uint64(1)) == ERR_ARG
    assert L.svm_spp_step(None, C.c_double(0.01), C.c_double(1.0), C.c_double(0.1), C.c_double(1.0), 1, None,
                          C.c_uint64(1)) == ERR_ARG
    cnt = C.c_int()
    assert L.svm_mlp_parameter_count(C.byref(cnt)) == 0 and cnt.value == 24 * 64 + 64 + 64 * 64 + 64 + 2 * 64 + 2
    assert L.svm_status_string(ERR_ARG) and L.svm_status_string(999)


def test_device_paths_fail_loudly_without_a_device(svm):
    """With no GPU the device entry points return an error that the Python classes raise; nothing
    falls back to host code (the host hull stays a separate, explicit entry point)."""
    if svm.device_count() > 0:
        pytest.skip("a device is present")
    pts = svm.random_cell_centres(3, 50)
    with pytest.raises(svm.SVMError):
        svm.Topology(pts, device=True)
    with pytest.raises(svm.SVMError):
        svm.sphericalVertexModel(50, svm.noiseSource())
    nl = svm.neighborList(1.0, 5.0)
    with pytest.raises(svm.SVMError):
        nl._ensure(10)
    assert svm.Topology(pts).nVertices == 96  # the explicit host builder


def test_neighbor_list_rejects_host_or_misshapen_points(svm):
    import torch
    nl = svm.neighborList(1.0, 5.0)
    for bad in (torch.zeros(10, 3, dtype=torch.float64), torch.zeros(10, 3, dtype=torch.float32),
                torch.zeros(10, 2, dtype=torch.float64), np.zeros((10, 3))):
        with pytest.raises(ValueError):
            nl.computeNeighborLists(bad)
