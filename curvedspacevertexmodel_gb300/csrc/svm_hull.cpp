// Randomised incremental 3-D convex hull with outside sets, plus the facet -> vertex-model
// topology builder.  See svm_hull.h for the contract this follows.
#include "svm_hull.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <random>

namespace svm {
namespace {

struct Face {
    int v[3];
    int nb[3];          // nb[i]: face across directed edge v[i] -> v[(i+1)%3]
    bool alive;
    std::vector<int> outside;  // unprocessed points strictly above this face
};

// Sign of the orientation of p relative to the plane through a, b, c (positive: p lies on
// the side the normal (b-a) x (c-a) points to).  Double evaluation with a relative filter;
// near-degenerate cases are re-evaluated in long double.
inline double orient(const double* P, int a, int b, int c, int p) {
    const double* A = P + 3 * a; const double* B = P + 3 * b;
    const double* C = P + 3 * c; const double* D = P + 3 * p;
    double bx = B[0] - A[0], by = B[1] - A[1], bz = B[2] - A[2];
    double cx = C[0] - A[0], cy = C[1] - A[1], cz = C[2] - A[2];
    double dx = D[0] - A[0], dy = D[1] - A[1], dz = D[2] - A[2];
    double nx = by * cz - bz * cy, ny = bz * cx - bx * cz, nz = bx * cy - by * cx;
    double det = nx * dx + ny * dy + nz * dz;
    double perm = (std::fabs(by * cz) + std::fabs(bz * cy)) * std::fabs(dx) +
                  (std::fabs(bz * cx) + std::fabs(bx * cz)) * std::fabs(dy) +
                  (std::fabs(bx * cy) + std::fabs(by * cx)) * std::fabs(dz);
    if (std::fabs(det) > 1e-13 * perm) return det;
    long double Bx = (long double)B[0] - A[0], By = (long double)B[1] - A[1], Bz = (long double)B[2] - A[2];
    long double Cx = (long double)C[0] - A[0], Cy = (long double)C[1] - A[1], Cz = (long double)C[2] - A[2];
    long double Dx = (long double)D[0] - A[0], Dy = (long double)D[1] - A[1], Dz = (long double)D[2] - A[2];
    long double d2 = (By * Cz - Bz * Cy) * Dx + (Bz * Cx - Bx * Cz) * Dy + (Bx * Cy - By * Cx) * Dz;
    return (double)d2;
}

}  // namespace

bool convexHullTriangles(const double* P, int n, std::vector<int>& triangles) {
    triangles.clear();
    if (n < 4) return false;
    // Initial tetrahedron: 0, the farthest point from 0, the point farthest from that line,
    // and the point farthest from that plane.
    auto d2 = [&](int i, int j) {
        double s = 0; for (int d = 0; d < 3; ++d) { double t = P[3 * i + d] - P[3 * j + d]; s += t * t; } return s;
    };
    int i0 = 0, i1 = -1, i2 = -1, i3 = -1;
    double best = 0;
    for (int i = 1; i < n; ++i) { double t = d2(i0, i); if (t > best) { best = t; i1 = i; } }
    if (i1 < 0) return false;
    best = 0;
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1) continue;
        double ux = P[3*i1]-P[3*i0], uy = P[3*i1+1]-P[3*i0+1], uz = P[3*i1+2]-P[3*i0+2];
        double vx = P[3*i]-P[3*i0], vy = P[3*i+1]-P[3*i0+1], vz = P[3*i+2]-P[3*i0+2];
        double cx = uy*vz-uz*vy, cy = uz*vx-ux*vz, cz = ux*vy-uy*vx;
        double t = cx*cx+cy*cy+cz*cz;
        if (t > best) { best = t; i2 = i; }
    }
    if (i2 < 0) return false;
    best = 0;
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1 || i == i2) continue;
        double t = std::fabs(orient(P, i0, i1, i2, i));
        if (t > best) { best = t; i3 = i; }
    }
    if (i3 < 0 || best == 0) return false;

    std::vector<Face> faces;
    faces.reserve(2 * (size_t)n + 16);
    auto addFace = [&](int a, int b, int c) {
        Face f; f.v[0] = a; f.v[1] = b; f.v[2] = c; f.nb[0] = f.nb[1] = f.nb[2] = -1; f.alive = true;
        faces.push_back(std::move(f));
        return (int)faces.size() - 1;
    };
    // Orient the tetrahedron so that every face normal points away from the fourth point.
    if (orient(P, i0, i1, i2, i3) > 0) std::swap(i1, i2);
    int t[4][3] = {{i0, i1, i2}, {i0, i3, i1}, {i1, i3, i2}, {i2, i3, i0}};
    for (auto& tri : t) addFace(tri[0], tri[1], tri[2]);
    // Link neighbours of the four faces by brute force.
    for (int f = 0; f < 4; ++f)
        for (int e = 0; e < 3; ++e) {
            int a = faces[f].v[e], b = faces[f].v[(e + 1) % 3];
            for (int g = 0; g < 4; ++g) {
                if (g == f) continue;
                for (int k = 0; k < 3; ++k)
                    if (faces[g].v[k] == b && faces[g].v[(k + 1) % 3] == a) faces[f].nb[e] = g;
            }
        }

    // Deterministic shuffled insertion order.
    std::vector<int> order;
    order.reserve(n);
    for (int i = 0; i < n; ++i)
        if (i != i0 && i != i1 && i != i2 && i != i3) order.push_back(i);
    std::mt19937_64 rng(0x5eed1234ULL);
    for (size_t i = order.size(); i > 1; --i) {
        size_t j = (size_t)(rng() % i);
        std::swap(order[i - 1], order[j]);
    }
    std::vector<int> rank(n, -1);
    for (size_t i = 0; i < order.size(); ++i) rank[order[i]] = (int)i;
    for (int p : order)
        for (int f = 0; f < 4; ++f)
            if (orient(P, faces[f].v[0], faces[f].v[1], faces[f].v[2], p) > 0) { faces[f].outside.push_back(p); break; }

    std::vector<int> owner(n, -1);  // face whose outside set currently holds the point
    for (int f = 0; f < 4; ++f) for (int p : faces[f].outside) owner[p] = f;

    std::vector<int> visibleMark(faces.capacity() + 8, 0);
    std::vector<int> stack, visible, newFaces;
    std::vector<int> startAt(n, -1);  // new face whose first horizon vertex is this point
    int stamp = 0;
    for (int p : order) {
        int f0 = owner[p];
        if (f0 < 0 || !faces[f0].alive) continue;  // inside the current hull
        ++stamp;
        if ((int)visibleMark.size() < (int)faces.size() + 8) visibleMark.resize(faces.size() * 2 + 8, 0);
        visible.clear(); stack.clear();
        stack.push_back(f0); visibleMark[f0] = stamp;
        // Horizon edges (a->b of a visible face whose neighbour is not visible).
        std::vector<std::array<int, 3>> horizon;  // a, b, hidden neighbour
        while (!stack.empty()) {
            int f = stack.back(); stack.pop_back();
            visible.push_back(f);
            for (int e = 0; e < 3; ++e) {
                int g = faces[f].nb[e];
                if (g < 0) return false;
                if (visibleMark[g] == stamp) continue;
                if (visibleMark[g] == -stamp) { horizon.push_back({faces[f].v[e], faces[f].v[(e + 1) % 3], g}); continue; }
                if (orient(P, faces[g].v[0], faces[g].v[1], faces[g].v[2], p) > 0) {
                    visibleMark[g] = stamp; stack.push_back(g);
                } else {
                    visibleMark[g] = -stamp;
                    horizon.push_back({faces[f].v[e], faces[f].v[(e + 1) % 3], g});
                }
            }
        }
        newFaces.clear();
        for (auto& h : horizon) {
            int a = h[0], b = h[1], g = h[2];
            int nf = addFace(a, b, p);
            if ((int)visibleMark.size() < (int)faces.size() + 8) visibleMark.resize(faces.size() * 2 + 8, 0);
            faces[nf].nb[0] = g;
            for (int k = 0; k < 3; ++k)
                if (faces[g].v[k] == b && faces[g].v[(k + 1) % 3] == a) faces[g].nb[k] = nf;
            if (startAt[a] != -1) return false;  // horizon is not a simple cycle
            startAt[a] = nf;
            newFaces.push_back(nf);
        }
        for (int nf : newFaces) {
            int b = faces[nf].v[1];
            int next = startAt[b];          // face (b, c, p)
            if (next < 0) return false;
            faces[nf].nb[1] = next;         // across b -> p
            faces[next].nb[2] = nf;         // across p -> b
        }
        for (int nf : newFaces) startAt[faces[nf].v[0]] = -1;
        // Re-home the outside points of the removed faces.
        for (int f : visible) {
            faces[f].alive = false;
            for (int q : faces[f].outside) {
                if (q == p) continue;
                owner[q] = -1;
                for (int nf : newFaces)
                    if (orient(P, faces[nf].v[0], faces[nf].v[1], faces[nf].v[2], q) > 0) {
                        faces[nf].outside.push_back(q); owner[q] = nf; break;
                    }
            }
            std::vector<int>().swap(faces[f].outside);
        }
    }
    (void)rank;
    for (auto& f : faces)
        if (f.alive) { triangles.push_back(f.v[0]); triangles.push_back(f.v[1]); triangles.push_back(f.v[2]); }
    // Euler check for a triangulated sphere whose vertices are all the input points.
    int nf = (int)triangles.size() / 3;
    std::vector<int> used(n, 0);
    for (int x : triangles) used[x] = 1;
    int nUsed = std::accumulate(used.begin(), used.end(), 0);
    if (nf != 2 * nUsed - 4) return false;
    return nUsed == n;
}

bool topologyFromTriangles(const double* points, int n, const std::vector<int>& triangles,
                           Topology& topo) {
    const int nf = (int)triangles.size() / 3;
    // Canonical facet form: smallest cell first (rotation keeps the CCW orientation), facets
    // sorted lexicographically.
    std::vector<std::array<int, 3>> F(nf);
    for (int f = 0; f < nf; ++f) {
        int a = triangles[3 * f], b = triangles[3 * f + 1], c = triangles[3 * f + 2];
        if (b < a && b < c) { int t = a; a = b; b = c; c = t; }
        else if (c < a && c < b) { int t = c; c = b; b = a; a = t; }
        F[f] = {a, b, c};
    }
    std::sort(F.begin(), F.end());
    // Incidence: for each cell, the facets that contain it and the corner it sits at.
    std::vector<int> off(n + 1, 0);
    for (auto& t : F) for (int k = 0; k < 3; ++k) off[t[k] + 1]++;
    for (int i = 0; i < n; ++i) off[i + 1] += off[i];
    std::vector<int> inc(off[n]), fill(off.begin(), off.end() - 1);
    for (int f = 0; f < nf; ++f) for (int k = 0; k < 3; ++k) inc[fill[F[f][k]]++] = f * 3 + k;
    // Facet containing directed edge u -> v (u at corner k, v at corner k+1).
    auto facetWithEdge = [&](int u, int v) -> int {
        for (int s = off[u]; s < off[u + 1]; ++s) {
            int f = inc[s] / 3, k = inc[s] % 3;
            if (F[f][(k + 1) % 3] == v) return f;
        }
        return -1;
    };

    topo.nCells = n;
    topo.nVertices = nf;
    topo.vertexPos.assign(3 * (size_t)nf, 0.0);
    topo.vertexCells.assign(3 * (size_t)nf, -1);
    topo.vertexNeighbors.assign(3 * (size_t)nf, -1);
    const double radius = std::sqrt(points[0] * points[0] + points[1] * points[1] + points[2] * points[2]);
    for (int f = 0; f < nf; ++f) {
        double c[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < 3; ++k)
            for (int d = 0; d < 3; ++d) c[d] += points[3 * F[f][k] + d];
        for (int d = 0; d < 3; ++d) c[d] = (1.0 / 3.0) * c[d];
        double nrm = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        for (int d = 0; d < 3; ++d) topo.vertexPos[3 * f + d] = (radius / nrm) * c[d];
        for (int k = 0; k < 3; ++k) {
            topo.vertexCells[3 * f + k] = F[f][k];
            int from = F[f][(k + 2) % 3], to = F[f][k];       // facet edge ending at corner k
            int g = facetWithEdge(to, from);
            if (g < 0) return false;
            topo.vertexNeighbors[3 * f + k] = g;
        }
    }
    // Rings: clockwise seen from outside, starting at the lowest-numbered facet.  From facet
    // (.., x, w, ..) the next facet clockwise around x is the one across the edge x -> w.
    topo.ringOffsets.assign(n + 1, 0);
    topo.ringVertices.clear();
    topo.ringVertices.reserve(2 * (size_t)nf + n);
    topo.maxRing = 0;
    for (int x = 0; x < n; ++x) {
        topo.ringOffsets[x] = (int)topo.ringVertices.size();
        int deg = off[x + 1] - off[x];
        if (deg < 3) return false;
        int start = nf;
        for (int s = off[x]; s < off[x + 1]; ++s) start = std::min(start, inc[s] / 3);
        int f = start, count = 0;
        do {
            topo.ringVertices.push_back(f);
            int k = 0;
            while (F[f][k] != x) ++k;
            int w = F[f][(k + 1) % 3];
            f = facetWithEdge(w, x);
            if (f < 0 || ++count > deg) return false;
        } while (f != start);
        if (count != deg) return false;
        topo.maxRing = std::max(topo.maxRing, deg);
    }
    topo.ringOffsets[n] = (int)topo.ringVertices.size();
    return true;
}

}  // namespace svm
