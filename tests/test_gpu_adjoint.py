"""GPU transpose of trilinear interpolation (_ffip.transpose) and the
sensitivity correlation, against numpy restatements of the reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def interpn_transpose_ref(gx, gy, gz, pt):
    """Sequential restatement of app/ffip.cpp:308-352 / include/utility.hpp:706-749."""
    nx, ny, nz = len(gx), len(gy), len(gz)
    dx = gx[1] - gx[0] if nx > 1 else 1.0
    dy = gy[1] - gy[0] if ny > 1 else 1.0
    dz = gz[1] - gz[0] if nz > 1 else 1.0
    out = np.zeros((nz, ny, nx))

    def axis(q, n):
        if n == 1:
            return [(0, 1.0)]
        if q <= 0:
            return [] if q <= -1 else [(0, 1 + q)]
        if q >= n - 1:
            return [] if q >= n else [(n - 1, n - q)]
        i = int(q)
        t = q - i
        return [(i + 1, t), (i, 1 - t)]

    for p in pt:
        for iz, wz in axis((p[2] - gz[0]) / dz, nz):
            for iy, wy in axis((p[1] - gy[0]) / dy, ny):
                for ix, wx in axis((p[0] - gx[0]) / dx, nx):
                    out[iz, iy, ix] += p[3] * wz * wy * wx
    return out


def test_transpose_matches_reference_restatement():
    from ffip_gb300 import native
    rng = np.random.default_rng(3)
    gx = np.linspace(-2, 3, 11); gy = np.linspace(0, 1, 5); gz = np.array([0.5])
    pt = np.stack([rng.uniform(-3, 4, 500), rng.uniform(-0.5, 1.5, 500), rng.uniform(0, 1, 500), rng.normal(size=500)], 1)
    got = native.transpose(gx, gy, gz, pt)
    ref = interpn_transpose_ref(gx, gy, gz, pt)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13)


def test_transpose_is_the_adjoint_of_trilinear_interpolation():
    """<interp(u) at the points, w> = <u, transpose(points, w)> for points
    inside the grid (the adjointness the reference checks by differences in
    scripts/transpose test.py)."""
    from scipy.interpolate import RegularGridInterpolator
    from ffip_gb300 import native
    rng = np.random.default_rng(5)
    gx = np.linspace(-1, 2, 13); gy = np.linspace(0, 1, 6); gz = np.linspace(0.5, 1.5, 4)
    n = 700
    xyz = np.stack([rng.uniform(-1, 2, n), rng.uniform(0, 1, n), rng.uniform(0.5, 1.5, n)], 1)
    w = rng.normal(size=n)
    u = rng.normal(size=(len(gz), len(gy), len(gx)))
    lhs = np.sum(w * RegularGridInterpolator((gz, gy, gx), u)(xyz[:, ::-1]))
    rhs = np.sum(u * native.transpose(gx, gy, gz, np.concatenate([xyz, w[:, None]], 1)))
    assert abs(lhs - rhs) <= 1e-12 * np.abs(w).sum() * np.abs(u).max()


def test_transpose_errors():
    from ffip_gb300 import native
    with pytest.raises(ValueError):
        native.transpose([0, 1], [0, 1], [0, 1], np.zeros((3, 3)))
    with pytest.raises(KeyError):
        native.transpose([], [0, 1], [0, 1], np.zeros((3, 4)))


def test_sensitivity_matches_numpy():
    import ctypes
    from ffip_gb300 import native
    lib = native.load()
    rng = np.random.default_rng(4)
    n = 300
    fwd = rng.normal(size=n) + 1j * rng.normal(size=n)
    adj = rng.normal(size=n) + 1j * rng.normal(size=n)
    deps = np.full(n, 11.0 + 0.0j)
    xyz = np.stack([rng.uniform(0, 2, n), rng.uniform(0, 2, n), rng.uniform(0, 1, n)], 1)
    f, norm = 0.1, 0.3 - 0.7j
    gx = np.linspace(0, 2, 9); gy = np.linspace(0, 2, 9); gz = np.linspace(0, 1, 3)
    se = np.real(2j * np.pi * f * fwd * adj * deps / norm)
    ref = interpn_transpose_ref(gx, gy, gz, np.concatenate([xyz, se[:, None]], 1))
    out = np.zeros((3, 9, 9))
    D = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.ascontiguousarray(np.stack([a.real, a.imag], 1)) for a in (fwd, adj, deps)]
    rc = lib.ffip_sensitivity(0.0, 2 * np.pi * f, norm.real, norm.imag, D(keep[0]), D(keep[1]), D(keep[2]), D(xyz), n,
                              D(gx), 9, D(gy), 9, D(gz), 3, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == 0
    np.testing.assert_allclose(out, ref, rtol=1e-10, atol=1e-12)


def to_convolve_ref(in1, in2, transpose=False):
    """Sequential restatement of app/ffip.cpp:222-306 (both filter axes
    indexed with the first half-width, as there)."""
    n0, n1 = in1.shape
    r0, r1 = in2.shape[0] // 2, in2.shape[1] // 2
    out = np.zeros_like(in1)
    for i in range(n0):
        for j in range(n1):
            l0, l1, u0, u1 = max(i - r0, 0), max(j - r1, 0), min(i + r0 + 1, n0), min(j + r1 + 1, n1)
            w = 0.0
            for m in range(l0, u0):
                for n in range(l1, u1):
                    w += in2[m - i + r0, n - j + r0]
            if not transpose:
                s = 0.0
                for m in range(l0, u0):
                    for n in range(l1, u1):
                        s += in1[m, n] * in2[m - i + r0, n - j + r0]
                out[i, j] = s / w
            else:
                for m in range(l0, u0):
                    for n in range(l1, u1):
                        out[m, n] += in1[i, j] * in2[m - i + r0, n - j + r0] / w
    return out


@pytest.mark.parametrize("transpose", [False, True])
def test_to_convolve_matches_reference_restatement(transpose):
    from ffip_gb300 import native
    rng = np.random.default_rng(11)
    a = rng.uniform(0, 1, size=(13, 17))
    f = rng.uniform(0.1, 1, size=(5, 5))
    got = (native.to_convolve_transpose if transpose else native.to_convolve)(a, f)
    np.testing.assert_allclose(got, to_convolve_ref(a, f, transpose), rtol=1e-12, atol=1e-14)


def test_to_convolve_transpose_is_the_adjoint():
    from ffip_gb300 import native
    rng = np.random.default_rng(12)
    a, b = rng.normal(size=(9, 11)), rng.normal(size=(9, 11))
    f = rng.uniform(0.1, 1, size=(3, 3))
    lhs = np.sum(native.to_convolve(a, f) * b)
    rhs = np.sum(a * native.to_convolve_transpose(b, f))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_to_convolve_errors():
    from ffip_gb300 import native
    with pytest.raises(KeyError):
        native.to_convolve(np.zeros((3, 3)), np.ones((2, 3)))
    with pytest.raises(native.FfipError, match="half-widths"):
        native.to_convolve(np.zeros((3, 3)), np.ones((3, 5)))
