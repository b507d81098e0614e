"""Host side of the self-propelled updater: the model's initial directors follow the reference
construction of sphericalVertexModel.cpp:58-70 on the seeded stream bit for bit against the oracle, and
are unit tangent vectors."""
import numpy as np

import oracle


def test_initial_directors_match_oracle():
    from curvedspacevertexmodel_gb300.model import random_cell_centres, random_vertex_directors
    from curvedspacevertexmodel_gb300 import Topology
    for seed, n in ((1137, 80), (7, 250)):
        centres = random_cell_centres(seed, n)
        topo = Topology(centres)
        dirs = random_vertex_directors(seed, n, topo.vertexPositions)
        R = np.sqrt(n / (4 * np.pi))
        om = oracle.OracleModel(topo.vertexPositions, topo.rings, topo.ringCounts, topo.vertexCells,
                                topo.vertexNeighbors, R)
        nz = oracle.OracleNoise(seed)
        assert np.array_equal(nz.cell_centres(n), centres)   # the stream up to the vertex directors
        om.init_directors(nz)
        assert np.array_equal(om.directors(), dirs)
        p = topo.vertexPositions / np.linalg.norm(topo.vertexPositions, axis=1, keepdims=True)
        assert np.abs(np.sum(dirs * p, axis=1)).max() < 1e-14
        assert np.abs(np.linalg.norm(dirs, axis=1) - 1).max() < 1e-14
