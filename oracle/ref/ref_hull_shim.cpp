// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// Replacement for the reference's CGAL-based initial topology
// (src/model/convexHullCGAL.cpp:82-186), which cannot be built here because CGAL is absent.
// It fills the reference's GPUArrays with the topology of svm_hull (the same hull code that
// initialises the product), following the contract of convexHullCGAL.cpp:
//   vertexPositions[nFaces], numVertexNeighs[nFaces] = 3, vertexNeighs / vertexCellNeighs with
//   Index2D(3, nFaces), numNeighs[n] = ring sizes, allNeighs with Index2D(maxDegree, n).
#include <stdexcept>
#include <vector>
#include "convexHullCGAL.h"
#include "svm_hull.h"

void convexHullCGALInterface::sphericalConvexHullForVertexModel(
    dVec* points, int n, GPUArray<int>& allNeighs, GPUArray<unsigned int>& numNeighs, Index2D& nidx,
    GPUArray<dVec>& vertexPositions, GPUArray<int>& vertexNeighs, GPUArray<int>& vertexCellNeighs,
    GPUArray<unsigned int>& numVertexNeighs, Index2D& vnidx) {
    std::vector<double> pts(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) pts[3 * i + d] = points[i].x[d];
    std::vector<int> tris;
    svm::Topology topo;
    if (!svm::convexHullTriangles(pts.data(), n, tris) || !svm::topologyFromTriangles(pts.data(), n, tris, topo))
        throw std::runtime_error("spherical hull failed");
    const int nf = topo.nVertices;
    vertexPositions.resize(nf);
    numVertexNeighs.resize(nf);
    vertexNeighs.resize(3 * nf);
    vertexCellNeighs.resize(3 * nf);
    vnidx = Index2D(3, nf);
    {
        ArrayHandle<dVec> vp(vertexPositions);
        ArrayHandle<unsigned int> vns(numVertexNeighs);
        ArrayHandle<int> vnset(vertexNeighs);
        ArrayHandle<int> vcset(vertexCellNeighs);
        for (int f = 0; f < nf; ++f) {
            for (int d = 0; d < 3; ++d) vp.data[f].x[d] = topo.vertexPos[3 * f + d];
            vns.data[f] = 3;
            for (int k = 0; k < 3; ++k) {
                vnset.data[vnidx(k, f)] = topo.vertexNeighbors[3 * f + k];
                vcset.data[vnidx(k, f)] = topo.vertexCells[3 * f + k];
            }
        }
    }
    if (numNeighs.getNumElements() < (unsigned)n) numNeighs.resize(n);
    const int W = topo.maxRing;
    allNeighs.resize(n * W);
    nidx = Index2D(W, n);
    ArrayHandle<unsigned int> nn(numNeighs);
    ArrayHandle<int> neighs(allNeighs);
    for (int c = 0; c < n; ++c) {
        int b = topo.ringOffsets[c], e = topo.ringOffsets[c + 1];
        nn.data[c] = (unsigned)(e - b);
        for (int k = 0; k < e - b; ++k) neighs.data[nidx(k, c)] = topo.ringVertices[b + k];
    }
}

void convexHullCGALInterface::sphericalConvexHull(dVec*, int, GPUArray<int>&, GPUArray<unsigned int>&, Index2D&) {
    throw std::runtime_error("sphericalConvexHull is not used on the vertex-model path");
}
