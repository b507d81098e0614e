// Spherical Delaunay triangulation (3-D convex hull of points on a sphere) and the
// vertex-model topology derived from it.
//
// This is the initialisation step of the spherical vertex model.  The reference builds it
// with CGAL::convex_hull_3 in convexHullCGALInterface::sphericalConvexHullForVertexModel
// (src/model/convexHullCGAL.cpp:82-186).  That routine fixes the contract this file
// follows:
//   * every hull facet (a Delaunay triangle of cell centres) is one vertex of the model;
//   * the vertex sits at radius * normalise(centroid of its three cell centres), the
//     centroid summed corner by corner and scaled by 1/3 (convexHullCGAL.cpp:67-80,118-127);
//   * vertex->cell slot k is the cell at facet corner k, walking the facet counter-clockwise
//     seen from outside, and vertex->vertex slot k is the facet across the facet edge that
//     ends at corner k (convexHullCGAL.cpp:137-149);
//   * the ring of a cell lists its facets clockwise seen from outside, which is the order of
//     CGAL's Halfedge_around_vertex_circulator (convexHullCGAL.cpp:170-185).  The included
//     angle of the reference treats det(prev, cur, next) > 0 as a reflex corner
//     (inc/sphericalDomain.h:114-133), so the clockwise order is load-bearing.
// CGAL's facet numbering and circulator start points are implementation details; this file
// fixes them canonically (facets sorted by their corner triple with the smallest cell first,
// each ring starting at its lowest-numbered facet), so the topology is a deterministic
// function of the input points.
#pragma once
#include <cstdint>
#include <vector>

namespace svm {

struct Topology {
    int nCells = 0;
    int nVertices = 0;
    int maxRing = 0;                       // largest ring (cell vertex count)
    std::vector<double> vertexPos;         // [3*nVertices] AoS x,y,z
    std::vector<int> vertexCells;          // [3*nVertices] vertex->cell
    std::vector<int> vertexNeighbors;      // [3*nVertices] vertex->vertex
    std::vector<int> ringOffsets;          // [nCells+1] CSR offsets into ringVertices
    std::vector<int> ringVertices;         // clockwise ring of each cell
};

// Triangles of the convex hull of points (CCW seen from outside), as cell-index triples.
// Returns false when the hull is degenerate (fewer than 4 non-coplanar points) or when the
// result fails the Euler/edge-pairing checks.
bool convexHullTriangles(const double* points, int n, std::vector<int>& triangles);

// Builds the vertex-model topology from hull triangles.  `points` are the cell centres; the
// vertex radius is |points[0]| as in convexHullCGAL.cpp:84.  Returns false on an invalid
// triangle set (an edge not shared by exactly two facets).
bool topologyFromTriangles(const double* points, int n, const std::vector<int>& triangles,
                           Topology& topo);

}  // namespace svm

// The C ABI's topology handle (svm_topology_*), filled by the host hull or the device hull.
struct svm_topology { svm::Topology t; };
