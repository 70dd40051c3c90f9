"""ffip_check_inside on the GPU against the oracle restatement of
_ffip.check_inside (app/ffip.cpp:353-387): bit-for-bit equal answers on
random, boundary and near-boundary points, polygons larger than one staged
chunk, and the planar_polygon density of the design scripts."""
import numpy as np
import pytest

from oracle import polygon as oracle

pytestmark = pytest.mark.gpu


def star_polygon(rng, m, r0=1.0):
    ang = np.sort(rng.uniform(0, 2 * np.pi, m))
    rad = r0 * rng.uniform(0.3, 1.0, m)
    return np.stack((rad * np.cos(ang), rad * np.sin(ang)), 1)


def boundary_points(rng, poly):
    q = [poly]
    a, b = poly, np.roll(poly, -1, axis=0)
    t = rng.uniform(size=(len(poly), 1))
    p = a + t * (b - a)
    q += [p, np.nextafter(p, p + 1), np.nextafter(p, p - 1), (a + b) / 2]
    return np.concatenate(q)


def test_cgal_manual_example():
    from ffip_gb300 import native
    poly = np.array([[0, 0], [5.1, 0], [1, 1], [0.5, 6]])
    got = native.check_inside(np.array([[0.5, 0.5], [1.5, 2.5], [2.5, 0.0]]), poly)
    assert got.tolist() == [True, False, False]


@pytest.mark.parametrize("m", [3, 5, 17, 200, 2047, 2048, 2049, 5000])
def test_random_star_polygons(m):
    from ffip_gb300 import native
    rng = np.random.default_rng(m)
    poly = star_polygon(rng, m, r0=3.0)
    q = np.concatenate((rng.uniform(-3.2, 3.2, (20000, 2)), boundary_points(rng, poly)))
    want = oracle.check_inside(q, poly)
    got = native.check_inside(q, poly)
    assert got.dtype == bool and got.shape == want.shape
    np.testing.assert_array_equal(got, want)
    # the closed ring the design scripts pass (first vertex repeated) and the
    # reversed orientation give the same answers
    np.testing.assert_array_equal(native.check_inside(q, np.vstack((poly, poly[:1]))), want)
    np.testing.assert_array_equal(native.check_inside(q, poly[::-1]), want)


def test_rectilinear_polygon_exact_edges():
    from ffip_gb300 import native
    # a rectilinear outline on a 1/8 grid: edge points are exactly representable
    poly = np.array([[0, 0], [4, 0], [4, 1], [2, 1], [2, 3], [4, 3], [4, 4], [0, 4]], float) * 0.125
    g = np.arange(-1, 34) / 64.0
    X, Y = np.meshgrid(g, g, indexing="ij")
    q = np.stack((X, Y), -1)                                  # (35, 35, 2): result (35, 35)
    want = oracle.check_inside(q, poly)
    got = native.check_inside(q, poly)
    assert got.shape == (35, 35)
    np.testing.assert_array_equal(got, want)
    assert want.any() and (~want).any()


def test_empty_and_degenerate_inputs():
    from ffip_gb300 import native
    q = np.random.default_rng(3).uniform(-1, 1, (100, 2))
    assert native.check_inside(np.zeros((0, 2)), star_polygon(np.random.default_rng(1), 8)).shape == (0,)
    assert not native.check_inside(q, np.zeros((0, 2))).any()
    assert not native.check_inside(q, np.array([[0.0, 0.0], [1.0, 1.0]])).any()


def test_large_query_set():
    from ffip_gb300 import native
    rng = np.random.default_rng(11)
    poly = star_polygon(rng, 64)
    q = rng.uniform(-1, 1, (1 << 20, 2))
    np.testing.assert_array_equal(native.check_inside(q, poly), oracle.check_inside(q, poly))


def test_planar_polygon_density():
    import ffip_gb300 as ffip
    # the bowtie of the reference's design scripts (two triangles and a bar),
    # given as three rings OR-ed together
    a, b, c, d = 30, 40, 50, 50

    class Multi:
        geoms = [np.array([(0, b), (c, b + d), (-c, b + d)], float), np.array([(0, -b), (c, -b - d), (-c, -b - d)], float),
                 np.array([(-a / 2, -b - d), (a / 2, -b - d), (a / 2, b + d), (-a / 2, b + d)], float)]

    f = ffip.planar_polygon(Multi(), center=ffip.Vector3(1.0, -2.0, 0.0), height=20)
    z, y, x = ffip.getgrid(ffip.Vector3(0, 0, 0), ffip.Vector3(120, 200, 40), ffip.Vector3(61, 101, 9))
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    pts = np.stack((Z, Y, X), -1)
    got = f(pts)
    xy = np.stack((X - 1.0, Y + 2.0), -1)
    want = np.zeros(X.shape, dtype=bool)
    for ring in Multi.geoms:
        want |= oracle.check_inside(xy, ring)
    want &= np.abs(Z) < 10
    np.testing.assert_array_equal(got, want * 1)
    assert got.sum() > 0
