"""ORACLE — test infrastructure, not the product.

CPU restatement of ``_ffip.check_inside`` (app/ffip.cpp:353-387).  The
reference builds a ``CGAL::Polygon_2`` over the Exact_predicates_inexact_
constructions kernel (CGAL >= 4.11, CMakeLists.txt:12) from the vertex pairs
and reports ``bounded_side(q) == ON_BOUNDED_SIDE`` for every query point.
CGAL is not in this image; its published semantics are restated instead: for a
simple polygon (its first vertex may be repeated at the end, as the closed
rings that ffip/geom.py:572-575 passes are), a point is on the bounded side
when it lies strictly inside -- not on an edge, not on a vertex.

Restatement: an exact crossing count along +x.  A point on an edge (exact
orientation 0 within the edge's bounding box) is on the boundary; otherwise
each edge whose end points straddle the point's y (one strictly above, the
other not) and that passes to the right of the point flips the parity.
Orientation signs come from float64 where the determinant is far from zero
relative to its terms (margin 1e-12, well beyond orient2d's rounding error of
about 3.3e-16) and from exact rational arithmetic (``fractions.Fraction``)
everywhere else.

Used only by tests/ as the checker of ``ffip_check_inside``.
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np


def _orient_exact(ax, ay, bx, by, cx, cy) -> int:
    F = Fraction
    d = (F(ax) - F(cx)) * (F(by) - F(cy)) - (F(ay) - F(cy)) * (F(bx) - F(cx))
    return (d > 0) - (d < 0)


def _orient(ax, ay, bx, by, cx, cy) -> np.ndarray:
    """Exact sign of (a - c) x (b - c) for arrays of points (int8)."""
    dl = (ax - cx) * (by - cy)
    dr = (ay - cy) * (bx - cx)
    det = dl - dr
    sure = np.abs(det) > 1e-12 * (np.abs(dl) + np.abs(dr))
    out = np.sign(det).astype(np.int8)
    for i in np.flatnonzero(~sure):
        out.flat[i] = _orient_exact(float(ax.flat[i]), float(ay.flat[i]), float(bx.flat[i]), float(by.flat[i]),
                                    float(cx.flat[i]), float(cy.flat[i]))
    return out


def check_inside(req_pts, poly_pts) -> np.ndarray:
    """bool array of shape req_pts.shape[:-1]: strictly inside the polygon."""
    q = np.asarray(req_pts, dtype=np.float64)
    p = np.asarray(poly_pts, dtype=np.float64).reshape(-1, 2)
    shape = q.shape[:-1]
    q = q.reshape(-1, 2)
    m = p.shape[0]
    inside = np.zeros(q.shape[0], dtype=bool)
    boundary = np.zeros(q.shape[0], dtype=bool)
    if m == 0:
        return inside.reshape(shape)
    qx, qy = q[:, 0], q[:, 1]
    for i in range(m):
        a, b = p[i], p[(i + 1) % m]
        straddle = (a[1] > qy) != (b[1] > qy)
        in_box = ((min(a[0], b[0]) <= qx) & (qx <= max(a[0], b[0])) & (min(a[1], b[1]) <= qy) & (qy <= max(a[1], b[1])))
        sel = np.flatnonzero(straddle | in_box)
        if sel.size == 0:
            continue
        o = _orient(np.full(sel.size, a[0]), np.full(sel.size, a[1]), np.full(sel.size, b[0]), np.full(sel.size, b[1]),
                    qx[sel], qy[sel])
        boundary[sel[(o == 0) & in_box[sel]]] = True
        right = (o > 0) if b[1] > a[1] else (o < 0)
        flip = sel[straddle[sel] & right]
        inside[flip] = ~inside[flip]
    return (inside & ~boundary).reshape(shape)
