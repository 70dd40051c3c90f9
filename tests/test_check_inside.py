"""check_inside (_ffip.check_inside, app/ffip.cpp:353-387): the oracle
restatement pinned to CGAL's documented example and to a fully rational
crossing count, and the host-side argument checks of the GPU entry point (no
GPU needed)."""
from fractions import Fraction

import numpy as np
import pytest

from oracle import polygon as oracle


def rational_inside(q, poly):
    """Strictly inside by a crossing count in exact rationals (no float)."""
    F = Fraction
    qx, qy = F(q[0]), F(q[1])
    m = len(poly)
    inside = False
    for i in range(m):
        ax, ay = F(poly[i][0]), F(poly[i][1])
        bx, by = F(poly[(i + 1) % m][0]), F(poly[(i + 1) % m][1])
        o = (ax - qx) * (by - qy) - (ay - qy) * (bx - qx)
        if o == 0 and min(ax, bx) <= qx <= max(ax, bx) and min(ay, by) <= qy <= max(ay, by):
            return False
        if (ay > qy) != (by > qy):
            # x of the crossing with y = qy
            xc = ax + (qy - ay) * (bx - ax) / (by - ay)
            if xc > qx:
                inside = not inside
    return inside


def star_polygon(rng, m, r0=1.0):
    ang = np.sort(rng.uniform(0, 2 * np.pi, m))
    rad = r0 * rng.uniform(0.3, 1.0, m)
    return np.stack((rad * np.cos(ang), rad * np.sin(ang)), 1)


def test_cgal_manual_example():
    # test/cgal_practice.cpp:22-31 of the reference: the CGAL manual's
    # bounded_side_2 example; (0.5, 0.5) inside, (1.5, 2.5) outside,
    # (2.5, 0) on the boundary
    poly = np.array([[0, 0], [5.1, 0], [1, 1], [0.5, 6]])
    got = oracle.check_inside(np.array([[0.5, 0.5], [1.5, 2.5], [2.5, 0.0]]), poly)
    assert got.tolist() == [True, False, False]


def test_square_closed_ring_and_concave():
    sq = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    q = np.array([[0.5, 0.5], [0, 0.5], [1, 1], [1.5, 0.5], [0.5, 0], [1e-300, 0.5], [-1e-300, 0.5]])
    want = [True, False, False, False, False, True, False]
    assert oracle.check_inside(q, sq).tolist() == want
    assert oracle.check_inside(q, np.vstack((sq, sq[:1]))).tolist() == want     # closed ring
    assert oracle.check_inside(q, sq[::-1]).tolist() == want                      # clockwise
    ell = np.array([[0, 0], [2, 0], [2, 1], [1, 1], [1, 2], [0, 2]], float)
    q = np.array([[0.5, 1.5], [1.5, 1.5], [1.5, 0.5], [1, 1.5], [1, 1]])
    assert oracle.check_inside(q, ell).tolist() == [True, False, True, False, False]
    # fewer than three distinct vertices: nothing is inside
    assert not oracle.check_inside(q, ell[:2]).any()
    assert oracle.check_inside(q, np.zeros((0, 2))).shape == (5,)


def test_oracle_matches_rational_crossing_count():
    rng = np.random.default_rng(7)
    for trial in range(12):
        poly = star_polygon(rng, int(rng.integers(3, 12)))
        q = [rng.uniform(-1.1, 1.1, 2) for _ in range(40)]
        q += [poly[i] for i in range(len(poly))]                                  # vertices
        for i in range(len(poly)):                                                 # on or next to edges
            a, b = poly[i], poly[(i + 1) % len(poly)]
            t = rng.uniform()
            p = a + t * (b - a)
            q += [p, np.nextafter(p, p + 1), np.nextafter(p, p - 1)]
        q = np.array(q)
        got = oracle.check_inside(q, poly)
        want = [rational_inside(x, poly) for x in q]
        assert got.tolist() == want, trial


def test_entry_point_argument_errors():
    from ffip_gb300 import native
    with pytest.raises(ValueError, match="ndim is not bigger than 1"):
        native.check_inside(np.zeros(2), np.zeros((3, 2)))
    with pytest.raises(ValueError, match="ndim is not bigger than 1"):
        native.check_inside(np.zeros((3, 2)), np.zeros(6))
    with pytest.raises(ValueError, match=r"req_pts.shape\[-1\] is not 2"):
        native.check_inside(np.zeros((3, 3)), np.zeros((3, 2)))
    with pytest.raises(ValueError, match=r"poly_pts.shape\[-1\] is not 2"):
        native.check_inside(np.zeros((3, 2)), np.zeros((3, 3)))
