"""ffip_transpose_noalloc (fixed device scratch, no allocation) against
ffip_transpose.  Kept in a file of its own that is collected last, so that it
runs both alone and after every other test in one process."""
import numpy as np
import pytest

from ffip_gb300 import native


def _case(seed, npts, nx, ny, nz):
    rng = np.random.default_rng(seed)
    gx = np.linspace(-2.0, 3.0, nx)
    gy = np.linspace(0.0, 1.5, ny)
    gz = np.linspace(-1.0, 1.0, nz) if nz > 1 else np.array([0.25])
    pt = np.stack([rng.uniform(-3, 4, npts), rng.uniform(-0.5, 2.0, npts), rng.uniform(-1.5, 1.5, npts),
                   rng.normal(size=npts)], 1)
    return gx, gy, gz, pt


@pytest.mark.gpu
def test_noalloc_matches_transpose_on_two_calls_in_a_row():
    # the second call is smaller and lands on a grid of another shape: any
    # output left in the scratch by the first call would show up in it
    for seed, npts, dims in ((1, 5000, (17, 9, 5)), (2, 700, (6, 11, 1))):
        gx, gy, gz, pt = _case(seed, npts, *dims)
        want = native.transpose(gx, gy, gz, pt)
        got = native.transpose_noalloc(gx, gy, gz, pt)
        assert got.shape == want.shape
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_noalloc_repeated_identical_calls_do_not_accumulate():
    gx, gy, gz, pt = _case(3, 2000, 8, 8, 8)
    first = native.transpose_noalloc(gx, gy, gz, pt)
    second = native.transpose_noalloc(gx, gy, gz, pt)
    np.testing.assert_allclose(second, first, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_noalloc_at_the_size_limit_and_empty_points():
    cap = 1 << 20
    nx = ny = 64
    nz = 64                     # 262144 output doubles
    npts = (cap - nx * ny * nz) // 4
    gx, gy, gz, pt = _case(4, npts, nx, ny, nz)
    np.testing.assert_allclose(native.transpose_noalloc(gx, gy, gz, pt), native.transpose(gx, gy, gz, pt),
                               rtol=1e-10, atol=1e-10)
    empty = native.transpose_noalloc(gx, gy, gz, np.zeros((0, 4)))
    assert not empty.any()


def test_noalloc_rejects_inputs_beyond_the_scratch():
    # rejected on the host before any CUDA call, so this needs no GPU
    lib = native.load()
    gx, gy, gz, pt = _case(5, 10, 128, 128, 65)    # 1064960 output doubles > 2**20
    with pytest.raises(native.FfipError, match="exceeds the fixed scratch"):
        native.transpose_noalloc(gx, gy, gz, pt, lib=lib)
    gx, gy, gz, pt = _case(6, 262100, 8, 8, 8)     # 4 * 262100 + 512 > 2**20
    with pytest.raises(native.FfipError, match="exceeds the fixed scratch"):
        native.transpose_noalloc(gx, gy, gz, pt, lib=lib)


def test_noalloc_rejects_a_point_count_whose_scratch_size_overflows():
    # npts = 2**62: 4 * npts wraps to 0 in 64 bits, so only the separate
    # npts bound stops it; the call must fail before it reads the points
    import ctypes
    lib = native.load()
    g = np.array([0.0])
    pt = np.zeros((1, 4))
    out = np.zeros(1)
    D = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    rc = lib.ffip_transpose_noalloc(D(g), 1, D(g), 1, D(g), 1, D(pt), 1 << 62, D(out))
    assert rc == -1
    assert "exceeds the fixed scratch" in lib.ffip_last_error().decode()
