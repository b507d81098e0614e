"""ORACLE — TEST INFRASTRUCTURE ONLY.

Initial vertex-model topology for the CPU oracle and the timed CPU reference leg, built without
any product code: scipy's qhull gives the hull triangles of the cell centres, and this module
restates the contract of convexHullCGALInterface::sphericalConvexHullForVertexModel
(src/model/convexHullCGAL.cpp:82-186) in numpy:
  * one vertex per facet at radius * normalise(centroid), radius = |points[0]| (84, 118-127);
  * vertex->cell slot k = facet corner k (CCW seen from outside), vertex->vertex slot k = the
    facet across the edge ending at corner k (137-149);
  * cell rings clockwise seen from outside (170-185).
The facet numbering and ring start follow the same canonical choice as the product's hull
(facets sorted by their corner triple with the smallest cell first; rings start at their
lowest-numbered facet), so both give identical arrays for the same points.
"""
from __future__ import annotations

import numpy as np


def hull_triangles(points: np.ndarray) -> np.ndarray:
    from scipy.spatial import ConvexHull
    tri = ConvexHull(points).simplices.astype(np.int64)
    a, b, c = points[tri[:, 0]], points[tri[:, 1]], points[tri[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(b - a, c - a), a) < 0
    tri[flip, 1], tri[flip, 2] = tri[flip, 2].copy(), tri[flip, 1].copy()
    return tri


def topology(points: np.ndarray, triangles: np.ndarray | None = None, width: int | None = None) -> dict:
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    tri = hull_triangles(pts) if triangles is None else np.asarray(triangles, dtype=np.int64)
    # canonical rotation (smallest corner first, orientation kept), then lexicographic order
    r = np.argmin(tri, axis=1)
    idx = (r[:, None] + np.arange(3)[None, :]) % 3
    F = np.take_along_axis(tri, idx, axis=1)
    order = np.lexsort((F[:, 2], F[:, 1], F[:, 0]))
    F = F[order]
    nf = F.shape[0]
    # vertex positions: centroid summed corner by corner, scaled by 1/3, renormalised
    radius = np.sqrt(pts[0, 0] * pts[0, 0] + pts[0, 1] * pts[0, 1] + pts[0, 2] * pts[0, 2])
    c = np.zeros((nf, 3))
    for k in range(3):
        c = c + pts[F[:, k]]
    c = (1.0 / 3.0) * c
    nrm = np.sqrt(c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1] + c[:, 2] * c[:, 2])
    vpos = (radius / nrm)[:, None] * c
    # directed edge (u -> v) -> facet
    key = {}
    for k in range(3):
        u, v = F[:, k], F[:, (k + 1) % 3]
        for f in range(nf):
            key[(int(u[f]), int(v[f]))] = f
    vcells = F.astype(np.int32)
    vnbrs = np.empty((nf, 3), dtype=np.int32)
    for f in range(nf):
        for k in range(3):
            frm, to = int(F[f, (k + 2) % 3]), int(F[f, k])
            vnbrs[f, k] = key[(to, frm)]
    # rings: clockwise from the lowest-numbered facet; next facet is across the edge x -> w
    first = np.full(n, nf, dtype=np.int64)
    np.minimum.at(first, F[:, 0], np.arange(nf))
    np.minimum.at(first, F[:, 1], np.arange(nf))
    np.minimum.at(first, F[:, 2], np.arange(nf))
    rings = []
    for x in range(n):
        f = int(first[x])
        ring = []
        while True:
            ring.append(f)
            k = int(np.nonzero(F[f] == x)[0][0])
            w = int(F[f, (k + 1) % 3])
            f = key[(w, x)]
            if f == first[x]:
                break
        rings.append(ring)
    counts = np.array([len(r) for r in rings], dtype=np.uint32)
    W = int(counts.max()) if width is None else width
    R = np.full((n, W), -1, dtype=np.int32)
    for x, ring in enumerate(rings):
        R[x, : len(ring)] = ring
    return dict(pos=vpos, rings=R, counts=counts, vcells=vcells, vnbrs=vnbrs, radius=float(radius))
