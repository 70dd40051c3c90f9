"""ctypes binding of the C ABI in include/ffip_gb300.h.

``load()`` returns the in-tree native library ffip_gb300/_lib/libffip_gb300.so
(building it first if needed) and raises if it cannot be built or loaded:
there is no CPU fallback.  ``NativeSim`` wraps one simulation handle;
``run_json`` is the one-call form of the reference's run_sim_json
(app/run_sim_json.cpp): config + datasets in, output datasets out.
"""
from __future__ import annotations

import ctypes
import json
import os
from typing import Dict, Optional, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


class FfipError(RuntimeError):
    pass


class Dataset(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("data", ctypes.POINTER(ctypes.c_double)), ("n", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("time_step", ctypes.c_int64), ("yee_cells", ctypes.c_int64), ("array_cells", ctypes.c_int64),
                ("dt", ctypes.c_double), ("dx", ctypes.c_double), ("bytes_per_step", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("fused", ctypes.c_int32), ("fp32", ctypes.c_int32),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64), ("pass_bytes_per_step", ctypes.c_double)]


EXPORTS = ["ffip_create", "ffip_step", "ffip_step_timed", "ffip_step_timed_pass", "ffip_run", "ffip_output_count",
           "ffip_output_group", "ffip_output_array", "ffip_set_density", "ffip_reset", "ffip_get_stats", "ffip_sync",
           "ffip_stream", "ffip_destroy", "ffip_last_error", "ffip_transpose", "ffip_sensitivity", "ffip_transpose_noalloc",
           "ffip_set_source_data", "ffip_to_convolve", "ffip_check_inside", "ffip_flux", "ffip_media_info"]


def _declare(lib):
    P, D, U64, I64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_uint64, ctypes.c_int64
    lib.ffip_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(Dataset), U64, ctypes.POINTER(P)]
    lib.ffip_step.argtypes = [P, I64]
    lib.ffip_step_timed.argtypes = [P, I64, ctypes.POINTER(ctypes.c_double)]
    lib.ffip_step_timed_pass.argtypes = [P, I64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.ffip_run.argtypes = [P, ctypes.c_char_p]
    lib.ffip_output_count.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    lib.ffip_output_group.argtypes = [P, ctypes.c_int, ctypes.c_char_p, U64]
    lib.ffip_output_array.argtypes = [P, ctypes.c_int, ctypes.c_char_p, D, U64, ctypes.POINTER(U64), ctypes.POINTER(ctypes.c_int)]
    lib.ffip_set_density.argtypes = [P, ctypes.c_char_p, D, U64]
    lib.ffip_set_source_data.argtypes = [P, ctypes.POINTER(Dataset), U64]
    lib.ffip_reset.argtypes = [P]
    lib.ffip_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
    lib.ffip_sync.argtypes = [P]
    lib.ffip_stream.argtypes = [P]
    lib.ffip_stream.restype = P
    lib.ffip_destroy.argtypes = [P]
    lib.ffip_last_error.restype = ctypes.c_char_p
    lib.ffip_transpose.argtypes = [D, U64, D, U64, D, U64, D, U64, D]
    lib.ffip_transpose_noalloc.argtypes = [D, U64, D, U64, D, U64, D, U64, D]
    lib.ffip_to_convolve.argtypes = [D, U64, U64, D, U64, U64, D, ctypes.c_int]
    lib.ffip_check_inside.argtypes = [D, U64, D, U64, ctypes.POINTER(ctypes.c_uint8)]
    lib.ffip_media_info.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)]
    lib.ffip_flux.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p, D, U64, D, U64, D, U64, D, D, U64, D]
    lib.ffip_sensitivity.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, D, D, D, D, U64,
                                     D, U64, D, U64, D, U64, D]
    for f in EXPORTS:
        if f not in ("ffip_stream", "ffip_last_error"):
            getattr(lib, f).restype = ctypes.c_int
    return lib


_lib = None


def lib_path() -> str:
    return os.path.join(_HERE, "_lib", "libffip_gb300.so")


def load(path: Optional[str] = None):
    """Loads (building if stale) the native library; raises FfipError if that fails."""
    global _lib
    if path is not None:
        return _declare(ctypes.CDLL(path))
    if _lib is None:
        try:
            from . import build as _build
            p = _build.build()
        except Exception as e:  # no silent fallback: the CUDA library is the product
            raise FfipError("cannot build the ffip_gb300 CUDA library: %s" % e) from e
        _lib = _declare(ctypes.CDLL(p))
    return _lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class NativeSim:
    """One simulation handle (ffip_create ... ffip_destroy)."""

    def __init__(self, config: dict, datasets: Optional[Dict[str, np.ndarray]] = None, lib=None):
        self.lib = lib if lib is not None else load()
        self._arrays = []
        ds = datasets or {}
        arr = (Dataset * max(1, len(ds)))()
        for i, (k, v) in enumerate(ds.items()):
            a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
            self._arrays.append(a)
            arr[i] = Dataset(k.encode(), _dptr(a), a.size)
        h = ctypes.c_void_p()
        self._check(self.lib.ffip_create(json.dumps(config).encode(), arr, len(ds), ctypes.byref(h)))
        self.h = h
        self.config = config

    def _check(self, rc):
        if rc != 0:
            raise FfipError("ffip error %d: %s" % (rc, self.lib.ffip_last_error().decode(errors="replace")))

    def step(self, n: int):
        self._check(self.lib.ffip_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        """Runs n steps; returns their device time in ms (CUDA events on the handle's stream)."""
        ms = ctypes.c_double()
        self._check(self.lib.ffip_step_timed(self.h, int(n), ctypes.byref(ms)))
        return ms.value

    def step_timed_pass(self, n: int) -> Tuple[float, float]:
        """Runs n steps; returns (device time of the n steps, summed device
        time of their fused field passes), both in ms; the second is 0 for
        the separate H and E passes."""
        ms, pms = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.ffip_step_timed_pass(self.h, int(n), ctypes.byref(ms), ctypes.byref(pms)))
        return ms.value, pms.value

    def run(self, stop: Optional[dict] = None):
        self._check(self.lib.ffip_run(self.h, json.dumps(stop).encode() if stop is not None else None))

    def sync(self):
        self._check(self.lib.ffip_sync(self.h))

    def reset(self):
        self._check(self.lib.ffip_reset(self.h))

    def set_density(self, dataset: str, rho: np.ndarray):
        a = np.ascontiguousarray(np.asarray(rho, dtype=np.float64).ravel())
        self._check(self.lib.ffip_set_density(self.h, dataset.encode(), _dptr(a), a.size))

    def set_source_data(self, datasets: Dict[str, np.ndarray]):
        """New amplitude/phase datasets of inhomogeneous sources; resets the fields."""
        keep = []
        arr = (Dataset * max(1, len(datasets)))()
        for i, (k, v) in enumerate(datasets.items()):
            a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
            keep.append(a)
            arr[i] = Dataset(k.encode(), _dptr(a), a.size)
        self._check(self.lib.ffip_set_source_data(self.h, arr, len(datasets)))

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.ffip_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def flux(self, e1_group: str, h2_group: str, x, y, z, w, freqs) -> np.ndarray:
        """Poynting flux per frequency through the integration grid x * y * z
        with weights w[z][y][x], from two monitor groups on the device."""
        c = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())  # noqa: E731
        x, y, z, w, f = c(x), c(y), c(z), c(w), c(freqs)
        out = np.zeros(f.size)
        self._check(self.lib.ffip_flux(self.h, e1_group.encode(), h2_group.encode(), _dptr(x), x.size, _dptr(y), y.size,
                                       _dptr(z), z.size, _dptr(w), _dptr(f), f.size, _dptr(out)))
        return out

    def media_info(self):
        """(per-component hashes of the device material tables, whether the
        media were rasterised on the GPU)"""
        cs = (ctypes.c_uint64 * 6)()
        dev = ctypes.c_int32()
        self._check(self.lib.ffip_media_info(self.h, cs, ctypes.byref(dev)))
        return [int(v) for v in cs], bool(dev.value)

    def stream(self) -> int:
        return self.lib.ffip_stream(self.h) or 0

    def outputs(self) -> dict:
        n = ctypes.c_int()
        self._check(self.lib.ffip_output_count(self.h, ctypes.byref(n)))
        out = {}
        name = ctypes.create_string_buffer(4096)
        for g in range(n.value):
            self._check(self.lib.ffip_output_group(self.h, g, name, 4096))
            grp = {}
            for arr in ("real", "imag", "x", "y", "z", "f"):
                dims = (ctypes.c_uint64 * 4)()
                nd = ctypes.c_int()
                rc = self.lib.ffip_output_array(self.h, g, arr.encode(), None, 0, dims, ctypes.byref(nd))
                if rc == -3:
                    continue
                self._check(rc)
                shape = tuple(int(dims[i]) for i in range(nd.value))
                a = np.zeros(int(np.prod(shape)) if shape else 0, dtype=np.float64)
                self._check(self.lib.ffip_output_array(self.h, g, arr.encode(), _dptr(a), a.size, dims, ctypes.byref(nd)))
                grp[arr] = a.reshape(shape)
            out[name.value.decode()] = grp
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.ffip_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_json(config: dict, datasets: Optional[Dict[str, np.ndarray]] = None, lib=None) -> dict:
    """config + datasets -> {group: {array: ndarray}}, like run_sim_json."""
    with NativeSim(config, datasets, lib=lib) as s:
        s.run(config["stop condition"])
        return s.outputs()


def transpose(gx, gy, gz, pt, lib=None) -> np.ndarray:
    """_ffip.transpose (app/ffip.cpp:308-352) on the GPU."""
    L = lib if lib is not None else load()
    gx, gy, gz = (np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel()) for v in (gx, gy, gz))
    pt = np.ascontiguousarray(np.asarray(pt, dtype=np.float64))
    if gx.size < 1 or gy.size < 1 or gz.size < 1:
        raise KeyError("some grid size is 0")
    if pt.ndim != 2:
        raise KeyError("some dimensions are not right")
    if pt.shape[1] != 4:
        raise ValueError("shape(1) of pts is not 4")
    out = np.zeros((gz.size, gy.size, gx.size), dtype=np.float64)
    rc = L.ffip_transpose(_dptr(gx), gx.size, _dptr(gy), gy.size, _dptr(gz), gz.size, _dptr(pt), pt.shape[0], _dptr(out))
    if rc != 0:
        raise FfipError(L.ffip_last_error().decode())
    return out


def transpose_noalloc(gx, gy, gz, pt, lib=None) -> np.ndarray:
    """transpose() through ffip_transpose_noalloc: no device allocation, at
    most 4 * npts + nx * ny * nz = 2**20 doubles, calls on one device must
    not overlap."""
    L = lib if lib is not None else load()
    gx, gy, gz = (np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel()) for v in (gx, gy, gz))
    pt = np.ascontiguousarray(np.asarray(pt, dtype=np.float64))
    if pt.ndim != 2 or pt.shape[1] != 4:
        raise ValueError("pts must have shape (n, 4)")
    out = np.zeros((gz.size, gy.size, gx.size), dtype=np.float64)
    rc = L.ffip_transpose_noalloc(_dptr(gx), gx.size, _dptr(gy), gy.size, _dptr(gz), gz.size, _dptr(pt), pt.shape[0],
                                  _dptr(out))
    if rc != 0:
        raise FfipError(L.ffip_last_error().decode())
    return out


def _to_convolve(in1, in2, transpose, lib=None):
    L = lib if lib is not None else load()
    a = np.ascontiguousarray(np.asarray(in1, dtype=np.float64))
    f = np.ascontiguousarray(np.asarray(in2, dtype=np.float64))
    if a.ndim != 2 or f.ndim != 2:
        raise KeyError("dimensions are not 2")
    if f.shape[0] % 2 == 0 or f.shape[1] % 2 == 0:
        raise KeyError("filter shape is not odd")
    out = np.zeros(a.shape, dtype=np.float64)
    rc = L.ffip_to_convolve(_dptr(a), a.shape[0], a.shape[1], _dptr(f), f.shape[0], f.shape[1], _dptr(out),
                            1 if transpose else 0)
    if rc != 0:
        raise FfipError(L.ffip_last_error().decode())
    return out


def to_convolve(in1, in2, lib=None) -> np.ndarray:
    """_ffip.TO_convolve (app/ffip.cpp:222-261) on the GPU."""
    return _to_convolve(in1, in2, False, lib)


def check_inside(req_pts, poly_pts, lib=None) -> np.ndarray:
    """_ffip.check_inside (app/ffip.cpp:353-387) on the GPU: for points
    req_pts[..., 2], whether each lies strictly inside the polygon
    poly_pts[..., 2] (CGAL bounded_side == ON_BOUNDED_SIDE; points on the
    boundary are not inside).  Returns bool of shape req_pts.shape[:-1]; the
    same ValueErrors as the reference for bad shapes."""
    L = lib if lib is not None else load()
    q = np.ascontiguousarray(np.asarray(req_pts, dtype=np.float64))
    p = np.ascontiguousarray(np.asarray(poly_pts, dtype=np.float64))
    if q.ndim < 2 or p.ndim < 2:
        raise ValueError("ndim is not bigger than 1")
    if q.shape[-1] != 2:
        raise ValueError("req_pts.shape[-1] is not 2")
    if p.shape[-1] != 2:
        raise ValueError("poly_pts.shape[-1] is not 2")
    out = np.zeros(q.shape[:-1], dtype=np.uint8)
    rc = L.ffip_check_inside(_dptr(q), q.size // 2, _dptr(p), p.size // 2, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise FfipError(L.ffip_last_error().decode())
    return out.astype(bool)


def to_convolve_transpose(in1, in2, lib=None) -> np.ndarray:
    """_ffip.TO_convolve_transpose (app/ffip.cpp:263-306) on the GPU."""
    return _to_convolve(in1, in2, True, lib)

