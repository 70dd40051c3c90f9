"""ORACLE — test infrastructure, not the product.

CPU restatement of the reference's FDTD hot path: this module restates, in
numpy, the set-up that ``Simulation::init`` performs from a config.json
(src/simulation.cpp:127-188) and drives the stepping loops of oracle/step.c,
which restate src/fields.cpp, src/structure.cpp and src/dft.cpp.  It is used
only by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs,
always as the checker or the timed CPU baseline, never as the product.

Pinning: tests/test_oracle_golden.py checks this port against golden DFT
outputs produced by the reference's own sources compiled here
(oracle/Makefile.ref -> oracle/_ref/run_sim_json, fixtures in tests/golden/).

Interface::

    sim = OracleSim(config_dict, datasets={name: ndarray}, threads=1)
    sim.run(config_dict["stop condition"])      # or sim.run_steps(n)
    out = sim.outputs()     # {group: {"real","imag","x","y","z","f"}, ...}

Coordinates are the reference's doubled grid: integer coordinate = 2*x/dx,
component parity bits Ex=001 Ey=010 Ez=100 Hx=110 Hy=101 Hz=011
(include/utility.hpp:48-64).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from typing import Dict, List, Optional

import numpy as np

PI = 3.141592653589793e+00

CTYPES = {"Ex": 0b001, "Ey": 0b010, "Ez": 0b100, "Hx": 0b110, "Hy": 0b101, "Hz": 0b011,
          "Dx": 0b1001, "Dy": 0b1010, "Dz": 0b1100, "Bx": 0b1110, "By": 0b1101, "Bz": 0b1011}
E_CTYPES = (0b001, 0b010, 0b100)
H_CTYPES = (0b110, 0b101, 0b011)
BC_PEC, BC_PMC, BC_NONE, BC_SYNC, BC_PERIOD = 0, 1, 2, 3, 4

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_LIB_DIR, "libffip_oracle.so")


# ----------------------------------------------------------------------------
# build / load oracle/step.c
# ----------------------------------------------------------------------------
def build(force: bool = False) -> str:
    """Compile oracle/step.c into oracle/_build/libffip_oracle.so (gcc, OpenMP,
    no FMA contraction so results do not depend on the host ISA)."""
    src = os.path.join(_HERE, "step.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    os.makedirs(_LIB_DIR, exist_ok=True)
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11", src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.oracle_run_steps.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        _lib.oracle_run_steps.restype = ctypes.c_int
        _lib.oracle_struct_size.restype = ctypes.c_int
    return _lib


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_F64 = ctypes.c_double


class _MediumGroup(ctypes.Structure):
    _fields_ = [("npoints", _I64), ("npoles", _I64), ("c1", _P), ("c2", _P), ("c3", _P),
                ("points", _P), ("amp", _P), ("p", _P), ("p1", _P)]


class _DftUnit(ctypes.Structure):
    _fields_ = [("npoints", _I64), ("is_db", _I64), ("nfreq", _I64), ("index", _P), ("freqs", _P),
                ("re", _P), ("im", _P), ("buf", _P)]


class _Sim(ctypes.Structure):
    _fields_ = [("eh", _P), ("accdb", _P), ("size", _I64), ("strides", _I64 * 3), ("inv_dx", _F64), ("dt", _F64),
                ("pml", (_P * 3) * 2), ("npml", (_I64 * 3) * 2),
                ("curl", (_P * 3) * 2), ("ncurl", (_I64 * 3) * 2),
                ("g1", _P * 2), ("g2", _P * 2), ("ng1", _I64 * 2), ("ng2", _I64 * 2), ("max_end", _F64 * 2),
                ("groups", _P * 2), ("ngroups", _I64 * 2),
                ("dft", _P * 2), ("ndft", _I64 * 2),
                ("bc", (_I64 * 2) * 3), ("grid_p1", _I64 * 3), ("grid_p2", _I64 * 3), ("ghost_p1", _I64 * 3),
                ("dim", _I64 * 3), ("face_buf", _P), ("face_cap", _I64), ("time_step", _I64), ("nthreads", _I64)]


PML_DTYPE = np.dtype([("index", np.int64), ("phi1", np.float64), ("b1", np.float64), ("c1", np.float64),
                      ("inv_k1", np.float64), ("phi2", np.float64), ("b2", np.float64), ("c2", np.float64),
                      ("inv_k2", np.float64)])
DIPOLE_DTYPE = np.dtype([("index", np.int64), ("amp", np.float64), ("start_time", np.float64),
                         ("end_time", np.float64), ("width", np.float64)])
MPOINT_DTYPE = np.dtype([("index", np.int64), ("g_inf", np.float64)])


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0


# ----------------------------------------------------------------------------
# small helpers restating include/utility.hpp
# ----------------------------------------------------------------------------
def cround(x: float) -> float:
    """std::round: halves away from zero."""
    return math.copysign(math.floor(abs(x) + 0.5), x)


def nearest_int(x: int, S: int, T: int) -> int:
    """get_nearest_int<S,T>(int), include/utility.hpp:478-485."""
    return x + S if ((x & 1) ^ T) else x


def nearest_point(p, ctype: int, S: int):
    """get_nearest_point<S>, include/utility.hpp:501-534 (float input uses
    floor for S=-1 and ceil for S=+1, :488-498)."""
    out = []
    for d in range(3):
        v = p[d]
        if not isinstance(v, (int, np.integer)):
            v = int(math.floor(v)) if S == -1 else int(math.ceil(v))
        out.append(nearest_int(int(v), S, (ctype >> d) & 1))
    return out


def component_interior(p1, p2, ctype):
    """include/utility.hpp:537-543"""
    return nearest_point(p1, ctype, +1), nearest_point(p2, ctype, -1)


def component_closure(p1, p2, ctype):
    """include/utility.hpp:546-552"""
    return nearest_point(p1, ctype, -1), nearest_point(p2, ctype, +1)


def cdiv(a: int, b: int) -> int:
    """C integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def yee_points(p1, p2, stride=2):
    """Coordinates visited by Yee_Iterator (src/utility.cpp:71-125), x fastest;
    returns (X, Y, Z) int64 arrays."""
    lens = [cdiv(p2[d] - p1[d], stride) + 1 for d in range(3)]
    if min(lens) <= 0:
        e = np.zeros(0, np.int64)
        return e, e, e
    xs = p1[0] + stride * np.arange(lens[0], dtype=np.int64)
    ys = p1[1] + stride * np.arange(lens[1], dtype=np.int64)
    zs = p1[2] + stride * np.arange(lens[2], dtype=np.int64)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return X.ravel(), Y.ravel(), Z.ravel()


def is_e_point(ctype: int) -> bool:
    return bin(ctype & 0b111).count("1") == 1


def linspace(s: float, e: float, n: int) -> np.ndarray:
    """src/utility.cpp:304-314"""
    if n <= 1:
        return np.array([s], dtype=np.float64)
    stride = (e - s) / (n - 1)
    return np.array([s + i * stride for i in range(n)], dtype=np.float64)


def gaussian1(t, width):
    arg = t / width
    return arg * math.exp(-arg * arg / 2)


# ----------------------------------------------------------------------------
# media, include/medium.hpp + src/medium.cpp
# ----------------------------------------------------------------------------
class Sus:
    def __init__(self, a0, a1, b0, b1, b2):
        self.c = (float(a0), float(a1), float(b0), float(b1), float(b2))

    def __eq__(self, o):  # src/medium.cpp:18-21
        return self.c == o.c

    def abstract(self, dt):
        """Abstract_Susceptibility, src/medium.cpp:24-31"""
        a0, a1, b0, b1, b2 = self.c
        c0 = 2 * b2 + b1 * dt
        c1 = (4 * b2 - 2 * b0 * dt * dt) / c0
        c2 = (-2 * b2 + b1 * dt) / c0
        c3 = (2 * a0 * dt * dt) / c0
        return c1, c2, c3


def json2sus(j) -> Sus:
    """src/simulation.cpp:88-100, src/medium.cpp:98-118"""
    t = j["type"]
    if t == "Lorentz":
        w = 2 * PI * float(j["frequency"])
        return Sus(w * w, 0, w * w, 2 * PI * float(j["gamma"]), 1)
    if t == "Drude":
        w = 2 * PI * float(j["frequency"])
        return Sus(w * w, 0, 0, 2 * PI * float(j["gamma"]), 1)
    if t == "Deybe":
        return Sus(1, 0, 1, float(j["tau"]), 0)
    raise ValueError("Unknonw susceptibility")


class Medium:
    def __init__(self, eps=0.0, mu=0.0):
        self.epsilon = float(eps)
        self.mu = float(mu)
        self.e_sus: List[Sus] = []
        self.e_amp: List[float] = []
        self.m_sus: List[Sus] = []
        self.m_amp: List[float] = []


def json2medium(j) -> Medium:
    """src/simulation.cpp:58-81"""
    m = Medium(j["epsilon"], j["mu"])
    ec = float(j["electric conductivity"])
    if ec != 0:
        m.e_sus.append(Sus(1, 0, 0, 1, 0)); m.e_amp.append(ec)
    mc = float(j["magnetic conductivity"])
    if mc != 0:
        m.m_sus.append(Sus(1, 0, 0, 1, 0)); m.m_amp.append(mc)
    for s in j.get("electric susceptibility", []):
        m.e_sus.append(json2sus(s)); m.e_amp.append(float(s["amplitude"]))
    for s in j.get("magnetic susceptibility", []):
        m.m_sus.append(json2sus(s)); m.m_amp.append(float(s["amplitude"]))
    return m


class AbMedium:
    """Abstract_Medium: epsilon, mu and amplitudes over the pool."""

    def __init__(self, eps, mu, e_amp, m_amp):
        self.epsilon, self.mu = eps, mu
        self.e_amp = np.asarray(e_amp, dtype=np.float64)
        self.m_amp = np.asarray(m_amp, dtype=np.float64)


# ----------------------------------------------------------------------------
# 1-D..3-D linear interpolation with zero-padded extrapolation
# (include/utility.hpp:644-849), vectorised over query points
# ----------------------------------------------------------------------------
def _interp1_weights(q: np.ndarray, n: int):
    """Return (i0, w0, i1, w1) for one axis, matching interpn's branches."""
    q = np.asarray(q, dtype=np.float64)
    i0 = np.zeros(q.shape, np.int64); i1 = np.zeros(q.shape, np.int64)
    w0 = np.zeros(q.shape); w1 = np.zeros(q.shape)
    if n == 1:
        w0[:] = 1.0
        return i0, w0, i1, w1
    lo = q <= 0
    lo_in = lo & (q > -1)
    w0[lo_in] = q[lo_in] + 1
    hi = (~lo) & (q >= n - 1)
    hi_in = hi & (q < n)
    i0[hi_in] = n - 1
    w0[hi_in] = n - q[hi_in]
    mid = (~lo) & (~hi)
    idx = q[mid].astype(np.int64)
    tx = q[mid] - idx
    i0[mid] = idx + 1; w0[mid] = tx      # first term: tx * data[index+1]
    i1[mid] = idx; w1[mid] = 1 - tx      # second term: (1-tx) * data[index]
    return i0, w0, i1, w1


def interp3(data: np.ndarray, dims, zq, yq, xq) -> np.ndarray:
    """interpn<3>(dz, dy, dx)(data, zq, yq, xq), include/utility.hpp:670-697.
    The reference recurses z -> y -> x and forms tx*A + (1-tx)*B at each level;
    that order of operations is kept."""
    nz, ny, nx = dims
    d = np.asarray(data, dtype=np.float64).reshape(nz, ny, nx)
    zi = _interp1_weights(zq, nz); yi = _interp1_weights(yq, ny); xi = _interp1_weights(xq, nx)

    def lvl_x(iz, iy):
        a = xi[1] * d[iz, iy, xi[0]]
        if nx == 1:
            return d[iz, iy, 0] * np.ones_like(a)
        q = np.asarray(xq, dtype=np.float64)
        mid = (q > 0) & (q < nx - 1)
        out = a.copy()
        out[mid] = a[mid] + xi[3][mid] * d[iz, iy, xi[2]][mid]
        return out

    def lvl_y(iz):
        if ny == 1:
            return lvl_x(iz, 0)
        q = np.asarray(yq, dtype=np.float64)
        a = yi[1] * lvl_x(iz, yi[0])
        mid = (q > 0) & (q < ny - 1)
        out = a.copy()
        out[mid] = a[mid] + yi[3][mid] * lvl_x(iz, yi[2])[mid]
        return out

    if nz == 1:
        return lvl_y(0)
    q = np.asarray(zq, dtype=np.float64)
    a = zi[1] * lvl_y(zi[0])
    mid = (q > 0) & (q < nz - 1)
    out = a.copy()
    out[mid] = a[mid] + zi[3][mid] * lvl_y(zi[2])[mid]
    return out


def interp1_medium(vals: np.ndarray, q: np.ndarray) -> np.ndarray:
    """interpn<1> over an array of per-entry values (src/geometry.cpp:104-106)."""
    n = vals.shape[0]
    i0, w0, i1, w1 = _interp1_weights(q, n)
    w0b = w0.reshape(w0.shape + (1,) * (vals.ndim - 1))
    w1b = w1.reshape(w1.shape + (1,) * (vals.ndim - 1))
    out = w0b * vals[i0]
    if n > 1:
        q = np.asarray(q, dtype=np.float64)
        mid = (q > 0) & (q < n - 1)
        out[mid] = out[mid] + w1b[mid] * vals[i1][mid]
    return out


# ----------------------------------------------------------------------------
# the simulation set-up
# ----------------------------------------------------------------------------
class OracleSim:
    def __init__(self, config: dict, datasets: Optional[Dict[str, np.ndarray]] = None, threads: int = 1):
        self.cfg = config
        self.datasets = {k: np.asarray(v, dtype=np.float64).ravel() for k, v in (datasets or {}).items()}
        self.threads = int(threads)
        self._keep = []
        self._init()

    # -- Simulation::init, src/simulation.cpp:127-188
    def _init(self):
        c = self.cfg
        sc = float(c.get("courant number", 0.5))
        self.resolution = float(c["resolution"])
        self.dx = 1 / self.resolution
        self.dt = self.dx * sc
        self.dx2 = self.dx / 2
        self._set_size()
        self._read_bcs()
        self._set_grid()
        bg = json2medium(c["default material"]) if "default material" in c else Medium(1, 1)
        self.bg_medium = bg
        self.e_pool: List[Sus] = []
        self.m_pool: List[Sus] = []
        self._add_to_pool([bg])
        self._set_pmls(c.get("PML", []))
        self._set_geometry(c.get("geometry", []))
        self.geom_info = {}
        for req in c.get("geometry info request", []):
            self._geometry_info_request(req)
        self.dipoles = {0: {"g1": [], "g2": []}, 1: {"g1": [], "g2": []}}
        self.turnoff_time = 0.0
        for src in c.get("sources", []):
            t = src["type"]
            if t == "volume source":
                self._set_volume_source(src)
            elif t == "inhomogeneous source":
                self._set_inhom_source(src)
        self._set_fields_output(c.get("fields output", []))
        self._build_struct()

    def _set_size(self):
        """src/simulation.cpp:570-581"""
        self.sim_size = [float(v) for v in self.cfg["size"]]
        span = [int(cround(self.sim_size[d] / self.dx)) * 2 for d in range(3)]
        self.sim_p1 = [-cdiv(s, 2) for s in span]
        self.sim_p2 = [cdiv(s, 2) for s in span]

    def _read_bcs(self):
        """src/simulation.cpp:583-653"""
        self.bcs = [[BC_NONE, BC_NONE] for _ in range(3)]
        for s in self.cfg.get("symmetry", []):
            d = {"x": 0, "y": 1, "z": 2}.get(s["direction"])
            if d is None:
                continue
            self.sim_p1[d] = 0
            self.bcs[d][0] = BC_PMC if int(s["phase factor"]) == 1 else BC_PEC
        if "periodic" in self.cfg:
            pd = self.cfg["periodic"]
            for d in range(3):
                if int(pd[d]):
                    if self.bcs[d][0] in (BC_PMC, BC_PEC):
                        self.bcs[d][1] = self.bcs[d][0]
                    else:
                        self.bcs[d][0] = self.bcs[d][1] = BC_PERIOD

    def _set_grid(self):
        """src/simulation.cpp:525-568 for one rank; Yee3 src/utility.cpp:130-140"""
        self.sim_dim = [self.sim_p2[d] - self.sim_p1[d] + 1 for d in range(3)]
        self.grid_p1 = list(self.sim_p1)
        self.grid_p2 = [self.sim_p1[d] + self.sim_dim[d] - 1 for d in range(3)]
        self.ghost_p1 = [v - 1 for v in self.grid_p1]
        ghost_p2 = [v + 1 for v in self.grid_p2]
        self.dim = [ghost_p2[d] - self.ghost_p1[d] + 1 for d in range(3)]
        self.strides = [1, self.dim[0], self.dim[0] * self.dim[1]]
        self.size = self.dim[0] * self.dim[1] * self.dim[2]
        self.eh = np.zeros(self.size, np.float64)
        self.accdb = np.zeros(self.size, np.float64)

    def index(self, X, Y, Z):
        """Yee3::get_index_from_coord, src/utility.cpp:206-210"""
        return ((X - self.ghost_p1[0]) + (Y - self.ghost_p1[1]) * self.strides[1]
                + (Z - self.ghost_p1[2]) * self.strides[2])

    def is_inside(self, p) -> bool:
        return all(self.grid_p1[d] <= p[d] <= self.grid_p2[d] for d in range(3))

    def _add_to_pool(self, media):
        """Structure::add_to_material_pool, src/structure.cpp:95-124"""
        for m in media:
            for s in m.e_sus:
                if not any(s == q for q in self.e_pool):
                    self.e_pool.append(s)
            for s in m.m_sus:
                if not any(s == q for q in self.m_pool):
                    self.m_pool.append(s)

    def _abstract(self, m: Medium) -> AbMedium:
        """Structure::get_abstract_medium, src/structure.cpp:126-153"""
        ea = np.zeros(len(self.e_pool)); ma = np.zeros(len(self.m_pool))
        for s, a in zip(m.e_sus, m.e_amp):
            for j, q in enumerate(self.e_pool):
                if q == s:
                    ea[j] = a
                    break
        for s, a in zip(m.m_sus, m.m_amp):
            for j, q in enumerate(self.m_pool):
                if q == s:
                    ma[j] = a
                    break
        return AbMedium(m.epsilon, m.mu, ea, ma)

    # -- PML, src/simulation.cpp:655-726, src/fields.cpp:485-506
    def _set_pmls(self, pmls):
        k = [np.ones(self.sim_dim[d]) for d in range(3)]
        b = [np.zeros(self.sim_dim[d]) for d in range(3)]
        cc = [np.zeros(self.sim_dim[d]) for d in range(3)]
        dt = self.dt
        for p in pmls:
            thick = float(p["thickness"]); kmax = float(p["k max"]); smax = float(p["sigma max"])
            order = int(p["order"])
            dirs = [0, 1, 2]
            sides = [-1, 1]
            if "direction" in p:
                dirs = [{"x": 0, "y": 1, "z": 2}[p["direction"]]]
            if "side" in p:
                sides = [{"positive": 1, "negative": -1}[p["side"]]]

            def get_sigma(x):
                return math.pow(x / thick, order) * smax

            def get_k(x):
                return 1 + (kmax - 1) * math.pow(x / thick, order)

            def get_b(x):
                return math.exp(-get_sigma(x) / get_k(x) * dt)

            def get_c(x):
                return 1 / get_k(x) * (get_b(x) - 1)

            for d in dirs:
                for side in sides:
                    half = self.sim_size[d] / 2
                    for i in range(self.sim_p1[d], self.sim_p2[d] + 1):
                        if side == 1 and (i * self.dx2 >= half - thick):
                            x = i * self.dx2 - (half - thick)
                        elif side == -1 and (i * self.dx2 <= -half + thick):
                            x = -half + thick - i * self.dx2
                        else:
                            continue
                        j = i - self.sim_p1[d]
                        k[d][j] = get_k(x); b[d][j] = get_b(x); cc[d][j] = get_c(x)
        self.pml_k, self.pml_b, self.pml_c = k, b, cc
        # Fields::init / PML_init_helper, include/fields.hpp:233-262
        self.pml_lists = {0: [None] * 3, 1: [None] * 3}
        self.curl_lists = {0: [None] * 3, 1: [None] * 3}
        for ct in E_CTYPES + H_CTYPES:
            side = 0 if is_e_point(ct) else 1
            x3 = {0b001: 0, 0b010: 1, 0b100: 2, 0b110: 0, 0b101: 1, 0b011: 2}[ct]
            x1, x2 = (x3 + 1) % 3, (x3 + 2) % 3
            p1, p2 = component_interior(self.grid_p1, self.grid_p2, ct)
            X, Y, Z = yee_points(p1, p2)
            P = (X, Y, Z)
            idx = self.index(X, Y, Z)
            i1 = P[x1] - self.sim_p1[x1]
            i2 = P[x2] - self.sim_p1[x2]
            is_pml = (cc[x1][i1] != 0) | (cc[x2][i2] != 0)
            pts = np.zeros(int(is_pml.sum()), PML_DTYPE)
            pts["index"] = idx[is_pml]
            pts["b1"] = b[x1][i1[is_pml]]; pts["c1"] = cc[x1][i1[is_pml]]
            pts["inv_k1"] = 1 / k[x1][i1[is_pml]]
            pts["b2"] = b[x2][i2[is_pml]]; pts["c2"] = cc[x2][i2[is_pml]]
            pts["inv_k2"] = 1 / k[x2][i2[is_pml]]
            self.pml_lists[side][x3] = pts
            self.curl_lists[side][x3] = np.ascontiguousarray(idx[~is_pml], dtype=np.int64)

    # -- geometry, src/simulation.cpp:359-518, src/structure.cpp:155-249
    def _set_geometry(self, geoms):
        mats = []
        for g in geoms:
            if g["type"] != "two medium box":
                mats.append(json2medium(g["medium"]))
            else:
                mats.append(json2medium(g["medium1"]))
                mats.append(json2medium(g["medium2"]))
        self._add_to_pool(mats)
        self.e_ab_pool = [s.abstract(self.dt) for s in self.e_pool]
        self.m_ab_pool = [s.abstract(self.dt) for s in self.m_pool]
        objs = [self._build_geometry(g) for g in geoms]
        self.geom_objs = objs
        default = self._abstract(self.bg_medium)
        want_map = bool(self.cfg.get("geometry info request"))
        L = [self.grid_p2[d] - self.grid_p1[d] + 1 for d in range(3)]
        # geom_map over all points of the local grid, x fastest (only kept
        # when a geometry info request needs it)
        self.geom_map = np.full(L[0] * L[1] * L[2], -1, np.int32) if want_map else None
        groups = {0: {}, 1: {}}
        for ct in E_CTYPES + H_CTYPES:
            side = 0 if is_e_point(ct) else 1
            p1, p2 = component_interior(self.grid_p1, self.grid_p2, ct)
            lens = [cdiv(p2[d] - p1[d], 2) + 1 for d in range(3)]
            if min(lens) <= 0:
                continue
            axes = [p1[d] + 2 * np.arange(lens[d], dtype=np.int64) for d in range(3)]
            npool = len(self.e_pool) if side == 0 else len(self.m_pool)
            owner = np.full((lens[2], lens[1], lens[0]), -1, np.int32)
            owned_idx, owned_g, owned_amp = [], [], []
            for gi, obj in enumerate(objs):
                blo, bhi = obj.bbox()
                sl = []
                for d in range(3):
                    a = np.searchsorted(axes[d], math.floor(blo[d]) - 1, side="left")
                    b = np.searchsorted(axes[d], math.ceil(bhi[d]) + 1, side="right")
                    sl.append(slice(int(a), int(b)))
                if any(x.start >= x.stop for x in sl):
                    continue
                sub = owner[sl[2], sl[1], sl[0]]
                Z, Y, X = np.meshgrid(axes[2][sl[2]], axes[1][sl[1]], axes[0][sl[0]], indexing="ij")
                new = (sub < 0) & obj.inside(X, Y, Z)
                if not new.any():
                    continue
                sub[new] = gi
                Xn, Yn, Zn = X[new], Y[new], Z[new]
                eps, mu, ea, ma = obj.medium(Xn, Yn, Zn)
                g = np.broadcast_to(np.asarray(eps if side == 0 else mu, dtype=np.float64), Xn.shape)
                a = np.asarray(ea if side == 0 else ma, dtype=np.float64)
                if npool == 0:
                    a = np.zeros((Xn.size, 0))
                else:
                    a = np.broadcast_to(a.reshape((-1, npool)) if a.ndim > 1 else a.reshape((1, npool)), (Xn.size, npool))
                owned_idx.append(self.index(Xn, Yn, Zn)); owned_g.append(np.array(g)); owned_amp.append(np.array(a))
            if want_map:
                Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
                gm_idx = ((X - self.grid_p1[0]) + (Y - self.grid_p1[1]) * L[0]
                          + (Z - self.grid_p1[2]) * L[0] * L[1]).ravel()
                self.geom_map[gm_idx] = owner.ravel()
            # default-medium points
            Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
            free = (owner < 0).ravel()
            didx = self.index(X.ravel()[free], Y.ravel()[free], Z.ravel()[free])
            dg = np.full(didx.size, default.epsilon if side == 0 else default.mu)
            damp = np.broadcast_to((default.e_amp if side == 0 else default.m_amp).reshape(1, npool), (didx.size, npool))
            del X, Y, Z
            parts = [(didx, dg, damp)] + list(zip(owned_idx, owned_g, owned_amp))
            # group by non-zero pattern, tol 1e-4 (src/structure.cpp:256-264)
            for idx, g_inf, amps in parts:
                if idx.size == 0:
                    continue
                nz = np.abs(amps) > 1e-4
                masks = (nz * (1 << np.arange(npool, dtype=np.int64))).sum(axis=1) if npool else np.zeros(idx.size, np.int64)
                for m in np.unique(masks):
                    sel = masks == m
                    bits = [i for i in range(npool) if (int(m) >> i) & 1]
                    grp = groups[side].setdefault(int(m), {"bits": bits, "idx": [], "g": [], "amp": []})
                    grp["idx"].append(idx[sel]); grp["g"].append(g_inf[sel]); grp["amp"].append(amps[sel][:, bits])
        self.medium_groups = {0: [], 1: []}
        for side in (0, 1):
            pool = self.e_ab_pool if side == 0 else self.m_ab_pool
            for m, grp in groups[side].items():
                idx = np.concatenate(grp["idx"]); g = np.concatenate(grp["g"])
                amp = np.concatenate(grp["amp"], axis=0)
                order = np.argsort(idx, kind="stable")
                pts = np.zeros(idx.size, MPOINT_DTYPE)
                pts["index"] = idx[order]; pts["g_inf"] = g[order]
                bits = grp["bits"]
                self.medium_groups[side].append({
                    "points": pts, "amp": np.ascontiguousarray(amp[order]).ravel(),
                    "npoles": len(bits),
                    "c1": np.array([pool[i][0] for i in bits]), "c2": np.array([pool[i][1] for i in bits]),
                    "c3": np.array([pool[i][2] for i in bits]),
                    "p": np.zeros(idx.size * len(bits)), "p1": np.zeros(idx.size * len(bits))})

    def _build_geometry(self, g):
        """Simulation::build_geometry_from_json, src/simulation.cpp:402-518"""
        t = g["type"]
        dx2 = self.dx2
        if t in ("box", "sphere"):
            ab = self._abstract(json2medium(g["medium"]))
            center = [float(v) / dx2 for v in g["center"]]
            if t == "box":
                size = [float(v) / dx2 for v in g["size"]]
                return _Box(center, size, ab)
            return _Sphere(center, float(g["radius"]) / dx2, ab)
        if t == "two medium box":
            m1 = self._abstract(json2medium(g["medium1"]))
            m2 = self._abstract(json2medium(g["medium2"]))
            center = [float(v) / dx2 for v in g["center"]]
            size = [float(v) / dx2 for v in g["size"]]
            dim = [int(v) for v in g["dimension"]]
            rho = self.datasets[g["density dataset"]]
            return _TwoMediumBox(center, size, dim, m1, m2, rho)
        if t == "general medium box":
            med = json2medium(g["medium"])
            center = [float(v) / dx2 for v in g["center"]]
            size = [float(v) / dx2 for v in g["size"]]
            dim = [int(v) for v in g["dimension"]]
            rho = self.datasets[g["density dataset"]]
            rho_fun = self.datasets[g["density function dataset"]]
            eps = self.datasets[g["epsilon dataset"]]
            mu = self.datasets[g["mu dataset"]]
            ea = self.datasets[g["electric susceptibility amplitudes dataset"]]
            ma = self.datasets[g["magnetic susceptibility amplitudes dataset"]]
            funs = []
            ne, nm = len(med.e_sus), len(med.m_sus)
            for i in range(eps.size):
                m = Medium(eps[i], mu[i])
                m.e_sus = list(med.e_sus); m.m_sus = list(med.m_sus)
                m.e_amp = [float(ea[i * ne + j]) for j in range(ne)]
                m.m_amp = [float(ma[i * nm + j]) for j in range(nm)]
                funs.append(self._abstract(m))
            return _GeneralMediumBox(center, size, dim, rho, rho_fun, funs)
        raise ValueError("unknown geometry type " + t)

    # -- geometry info request, src/simulation.cpp:190-233
    def _geometry_info_request(self, req):
        ct = CTYPES[req["field component"]]
        gi = int(req["geometry index"])
        L = [self.grid_p2[d] - self.grid_p1[d] + 1 for d in range(3)]
        p1, p2 = component_interior(self.grid_p1, self.grid_p2, ct)
        X, Y, Z = yee_points(p1, p2)
        gm_idx = (X - self.grid_p1[0]) + (Y - self.grid_p1[1]) * L[0] + (Z - self.grid_p1[2]) * L[0] * L[1]
        sel = self.geom_map[gm_idx] == gi
        # the reference stores coord*dx2 into a std::vector<int> (truncation)
        tr = lambda v: np.trunc(v.astype(np.float64) * self.dx2)
        self.geom_info[req["output group"]] = {"x": tr(X[sel]), "y": tr(Y[sel]), "z": tr(Z[sel])}

    # -- sources, src/simulation.cpp:235-336, src/fields.cpp:183-232
    def _add_dipole(self, pos, ct, amp, start, freq, cutoff, kind):
        amp = -amp
        base = nearest_point(pos, ct, -1)
        sx = (pos[0] - base[0]) / 2; sy = (pos[1] - base[1]) / 2; sz = (pos[2] - base[2]) / 2
        w = [(1 - sx) * (1 - sy) * (1 - sz), sx * (1 - sy) * (1 - sz), (1 - sx) * sy * (1 - sz), sx * sy * (1 - sz),
             (1 - sx) * (1 - sy) * sz, sx * (1 - sy) * sz, (1 - sx) * sy * sz, sx * sy * sz]
        side = 0 if is_e_point(ct) else 1
        if kind == "g1":
            width = 1 / (2 * PI * freq)
        else:
            width = math.sqrt(2.0) / (2 * PI * freq)
        end = start + 2 * width * cutoff
        if end > self.turnoff_time:
            self.turnoff_time = end
        n = 0
        for k in (0, 2):
            for j in (0, 2):
                for i in (0, 2):
                    p = [base[0] + i, base[1] + j, base[2] + k]
                    # Gaussian1 keeps corners with weight > 1e-4 (src/fields.cpp:203);
                    # the Gaussian2 path of the reference mis-steps its weight
                    # index (src/fields.cpp:222-230); this restatement uses the
                    # per-corner weight for both.
                    if self.is_inside(p) and (kind == "g2" or w[n] > 1e-4):
                        idx = int(self.index(p[0], p[1], p[2]))
                        self.dipoles[side][kind].append((idx, amp * w[n], start, end, width))
                    n += 1

    def _set_volume_source(self, src):
        dx2 = self.dx2
        center = [float(v) / dx2 for v in src["center"]]
        size = [float(v) / dx2 for v in src["size"]]
        amp = float(src["amplitude"])
        ct = CTYPES[src["field component"]]
        f = src["function"]
        kind = {"Gaussian1": "g1", "Gaussian2": "g2"}.get(f["type"])
        freq, cutoff, st = float(f["frequency"]), float(f["cutoff"]), float(f["start time"])
        p1 = [center[d] - size[d] / 2 for d in range(3)]
        count = [int(cround(size[d] / 2)) for d in range(3)]
        dlen = [0.0] * 3
        for d in range(3):
            if count[d] != 0:
                dlen[d] = size[d] / count[d]
                amp *= dlen[d] / 2
        if kind is None:
            return
        for k in range(count[2] + 1):
            for j in range(count[1] + 1):
                for i in range(count[0] + 1):
                    p = [p1[0] + i * dlen[0], p1[1] + j * dlen[1], p1[2] + k * dlen[2]]
                    self._add_dipole(p, ct, amp, st, freq, cutoff, kind)

    def _set_inhom_source(self, src):
        dx2 = self.dx2
        center = [float(v) / dx2 for v in src["center"]]
        size = [float(v) / dx2 for v in src["size"]]
        dim = [int(v) for v in src["dimension"]]
        amp = self.datasets[src["amplitude dataset"]]
        phase = self.datasets[src["phase dataset"]]
        ct = CTYPES[src["field component"]]
        fcen = float(src["frequency"])
        f = src["function"]
        kind = {"Gaussian1": "g1", "Gaussian2": "g2"}.get(f["type"])
        freq, cutoff, st = float(f["frequency"]), float(f["cutoff"]), float(f["start time"])
        p1 = [center[d] - size[d] / 2 for d in range(3)]
        dlen = [size[d] / (dim[d] - 1) if dim[d] > 1 else 0.0 for d in range(3)]
        if kind is None:
            return
        n = 0
        for k in range(dim[2]):
            for j in range(dim[1]):
                for i in range(dim[0]):
                    p = [p1[0] + i * dlen[0], p1[1] + j * dlen[1], p1[2] + k * dlen[2]]
                    self._add_dipole(p, ct, float(amp[n]), st - phase[n] / (2 * PI * fcen), freq, cutoff, kind)
                    n += 1

    # -- DFT, src/simulation.cpp:103-124, src/dft.cpp:6-25,163-192,253-271
    def _set_fields_output(self, outs):
        self.dft_units = []      # registration order per side kept in .side
        self.dft_requests = []
        for o in outs:
            if o["type"] != "volume fields dft":
                continue
            center = [float(v) / self.dx2 for v in o["center"]]
            size = [float(v) / self.dx2 for v in o["size"]]
            freqs = [float(v) for v in o["frequency"]]
            ct = CTYPES[o["field component"]]
            p1 = [center[d] - size[d] / 2 for d in range(3)]
            p2 = [center[d] + size[d] / 2 for d in range(3)]
            c1, c2 = component_closure(p1, p2, ct)
            unit = None
            for u in self.dft_units:
                if u["ctype"] == ct and u["p1"] == c1 and u["p2"] == c2:
                    unit = u
                    break
            if unit is None:
                unit = {"ctype": ct, "p1": c1, "p2": c2, "freqs": [],
                        "dim": [cdiv(c2[d] - c1[d], 2) + 1 for d in range(3)]}
                gp1, gp2 = self.grid_p1, self.grid_p2
                if all(c1[d] <= gp2[d] and gp1[d] <= c2[d] for d in range(3)):
                    q1 = [max(c1[d], gp1[d]) for d in range(3)]
                    q2 = [min(c2[d], gp2[d]) for d in range(3)]
                    l1, l2 = component_interior(q1, q2, ct)
                    unit["p1_local"], unit["p2_local"] = l1, l2
                    X, Y, Z = yee_points(l1, l2)
                    unit["index"] = np.ascontiguousarray(self.index(X, Y, Z), dtype=np.int64)
                    unit["local_dim"] = [cdiv(l2[d] - l1[d], 2) + 1 for d in range(3)]
                else:
                    unit["p1_local"] = c1
                    unit["index"] = np.zeros(0, np.int64)
                    unit["local_dim"] = [0, 0, 0]
                self.dft_units.append(unit)
            unit["freqs"].extend(freqs)
            self.dft_requests.append({"unit": unit, "freqs": freqs, "group": o["output group"],
                                      "closure": (c1, c2)})
        for u in self.dft_units:
            u["freqs"] = np.array(sorted(set(u["freqs"])), dtype=np.float64)
            n = u["index"].size
            u["re"] = np.zeros(n * u["freqs"].size)
            u["im"] = np.zeros(n * u["freqs"].size)
            u["buf"] = np.zeros(n)

    # -- hand the arrays to oracle/step.c
    def _build_struct(self):
        s = _Sim()
        K = self._keep
        s.eh = _ptr(self.eh); s.accdb = _ptr(self.accdb); s.size = self.size
        for d in range(3):
            s.strides[d] = self.strides[d]
        s.inv_dx = 1 / self.dx
        s.dt = self.dt
        for side in (0, 1):
            for d in range(3):
                pl = self.pml_lists[side][d]; cl = self.curl_lists[side][d]
                K += [pl, cl]
                s.pml[side][d] = _ptr(pl); s.npml[side][d] = pl.size
                s.curl[side][d] = _ptr(cl); s.ncurl[side][d] = cl.size
            g1 = np.array(self.dipoles[side]["g1"], dtype=DIPOLE_DTYPE) if self.dipoles[side]["g1"] else np.zeros(0, DIPOLE_DTYPE)
            g2 = np.array(self.dipoles[side]["g2"], dtype=DIPOLE_DTYPE) if self.dipoles[side]["g2"] else np.zeros(0, DIPOLE_DTYPE)
            K += [g1, g2]
            s.g1[side] = _ptr(g1); s.ng1[side] = g1.size
            s.g2[side] = _ptr(g2); s.ng2[side] = g2.size
            ends = [e[3] for e in self.dipoles[side]["g1"] + self.dipoles[side]["g2"]]
            s.max_end[side] = max(ends) if ends else 0.0
            grps = (_MediumGroup * max(1, len(self.medium_groups[side])))()
            for i, g in enumerate(self.medium_groups[side]):
                K += [g["points"], g["amp"], g["c1"], g["c2"], g["c3"], g["p"], g["p1"]]
                grps[i] = _MediumGroup(g["points"].size, g["npoles"], _ptr(g["c1"]), _ptr(g["c2"]), _ptr(g["c3"]),
                                       _ptr(g["points"]), _ptr(g["amp"]), _ptr(g["p"]), _ptr(g["p1"]))
            K.append(grps)
            s.groups[side] = ctypes.addressof(grps); s.ngroups[side] = len(self.medium_groups[side])
            units = [u for u in self.dft_units if (0 if is_e_point(u["ctype"]) else 1) == side]
            arr = (_DftUnit * max(1, len(units)))()
            for i, u in enumerate(units):
                arr[i] = _DftUnit(u["index"].size, 1 if u["ctype"] > 7 else 0, u["freqs"].size, _ptr(u["index"]),
                                  _ptr(u["freqs"]), _ptr(u["re"]), _ptr(u["im"]), _ptr(u["buf"]))
            K.append(arr)
            s.dft[side] = ctypes.addressof(arr); s.ndft[side] = len(units)
        for d in range(3):
            s.bc[d][0] = self.bcs[d][0]; s.bc[d][1] = self.bcs[d][1]
            s.grid_p1[d] = self.grid_p1[d]; s.grid_p2[d] = self.grid_p2[d]
            s.ghost_p1[d] = self.ghost_p1[d]; s.dim[d] = self.dim[d]
        L = [self.grid_p2[d] - self.grid_p1[d] + 1 for d in range(3)]
        cap = max(L[0] * L[1], L[1] * L[2], L[0] * L[2])
        self.face_buf = np.zeros(4 * cap)
        s.face_buf = _ptr(self.face_buf); s.face_cap = cap
        s.time_step = 0
        s.nthreads = self.threads
        self._s = s

    # ------------------------------------------------------------------
    @property
    def time_step(self) -> int:
        return int(self._s.time_step)

    def run_steps(self, n: int):
        _load().oracle_run_steps(ctypes.byref(self._s), int(n))

    def steps_until(self, t: float) -> int:
        """Number of loop iterations of run_until_time (src/simulation.cpp:773)."""
        n = self.time_step
        while n * self.dt < t:
            n += 1
        return n - self.time_step

    def interp_eh(self, pos, ct) -> float:
        """Yee3::interp on eh, include/utility.hpp:983-1022 (pos in doubled units)."""
        base = nearest_point(pos, ct, -1)
        res = 0.0
        if all(self.grid_p1[d] <= base[d] and base[d] + 2 <= self.grid_p2[d] for d in range(3)):
            inside_all = True
        elif all(base[d] <= self.grid_p2[d] and self.grid_p1[d] <= base[d] + 2 for d in range(3)):
            inside_all = False
        else:
            return 0.0
        sx = (pos[0] - base[0]) / 2; sy = (pos[1] - base[1]) / 2; sz = (pos[2] - base[2]) / 2
        w = [(1 - sx) * (1 - sy) * (1 - sz), sx * (1 - sy) * (1 - sz), (1 - sx) * sy * (1 - sz), sx * sy * (1 - sz),
             (1 - sx) * (1 - sy) * sz, sx * (1 - sy) * sz, (1 - sx) * sy * sz, sx * sy * sz]
        n = 0
        for k in (0, 2):
            for j in (0, 2):
                for i in (0, 2):
                    p = [base[0] + i, base[1] + j, base[2] + k]
                    if inside_all or self.is_inside(p):
                        res += self.eh[int(self.index(p[0], p[1], p[2]))] * w[n]
                    n += 1
        return res

    def run(self, stop: dict):
        """Simulation::run, src/simulation.cpp:903-958"""
        t = stop["type"]
        if t == "time":
            self.run_steps(self.steps_until(float(stop["time"])))
            return
        if t == "decay":
            pt = [float(v) / self.dx2 for v in stop["position"]]
            ct = CTYPES[stop["field component"]]
            interval = float(stop["time interval examined"]); decay_by = float(stop["decayed by"])
            mx = 0.0
            while self.time_step * self.dt < self.turnoff_time:
                self.run_steps(1)
                v = self.interp_eh(pt, ct) ** 2
                mx = max(mx, v)
            ext = 1
            while True:
                cur = 0.0
                while self.time_step * self.dt < self.turnoff_time + ext * interval:
                    self.run_steps(1)
                    v = self.interp_eh(pt, ct)
                    v = v * v
                    if v > cur:
                        cur = v
                ext += 1
                if cur > mx:
                    mx = cur
                if not (cur / mx > decay_by):
                    return
        # DFT steady state, src/simulation.cpp:782-842
        center = [float(v) for v in stop["center"]]; size = [float(v) for v in stop["size"]]
        ct = CTYPES[stop["field component"]]
        interval = float(stop["time interval examined"]); var = float(stop["variation"])
        freq = float(stop["frequency"])
        p1 = [(center[d] - size[d] / 2) / self.dx2 for d in range(3)]
        p2 = [(center[d] + size[d] / 2) / self.dx2 for d in range(3)]
        c1, c2 = component_closure(p1, p2, ct)
        unit = next((u for u in self.dft_units if u["ctype"] == ct and u["p1"] == c1 and u["p2"] == c2), None)
        if unit is None:
            raise RuntimeError("dft is not registered")
        fi = np.searchsorted(unit["freqs"], freq)
        if fi >= unit["freqs"].size or unit["freqs"][fi] != freq:
            raise RuntimeError("frequency is not registered")
        while self.time_step * self.dt < self.turnoff_time:
            self.run_steps(1)
        ext = 1
        n = unit["index"].size
        while True:
            mx = np.finfo(np.float64).tiny; mn = np.finfo(np.float64).max
            while self.time_step * self.dt < self.turnoff_time + ext * interval:
                self.run_steps(1)
                re = unit["re"][fi * n:(fi + 1) * n]; im = unit["im"][fi * n:(fi + 1) * n]
                nrm = 0.0
                for a, b in zip(re, im):
                    nrm += a * a + b * b
                mx = max(mx, nrm); mn = min(mn, nrm)
            ext += 1
            if not ((mx - mn) / mx > var):
                return

    def outputs(self) -> dict:
        """DFT_Hub::output_fields_collective (src/dft.cpp:273-320) and the
        geometry info groups (src/simulation.cpp:221-231)."""
        out = {}
        for r in self.dft_requests:
            u = r["unit"]
            c1, c2 = r["closure"]
            dim = u["dim"]
            nf = len(r["freqs"])
            re = np.zeros((nf, dim[2], dim[1], dim[0])); im = np.zeros_like(re)
            n = u["index"].size
            if n:
                off = [cdiv(u["p1_local"][d] - c1[d], 2) for d in range(3)]
                ld = u["local_dim"]
                for i, f in enumerate(r["freqs"]):
                    fi = int(np.searchsorted(u["freqs"], f))
                    if fi >= u["freqs"].size or u["freqs"][fi] != f:
                        raise RuntimeError("Frequencies not registered")
                    blk = (slice(off[2], off[2] + ld[2]), slice(off[1], off[1] + ld[1]), slice(off[0], off[0] + ld[0]))
                    re[(i,) + blk] = u["re"][fi * n:(fi + 1) * n].reshape(ld[2], ld[1], ld[0])
                    im[(i,) + blk] = u["im"][fi * n:(fi + 1) * n].reshape(ld[2], ld[1], ld[0])
            ph1 = [c1[d] * (self.dx / 2) for d in range(3)]
            ph2 = [c2[d] * (self.dx / 2) for d in range(3)]
            out[r["group"]] = {"real": re, "imag": im, "x": linspace(ph1[0], ph2[0], dim[0]),
                               "y": linspace(ph1[1], ph2[1], dim[1]), "z": linspace(ph1[2], ph2[2], dim[2]),
                               "f": np.array(r["freqs"], dtype=np.float64)}
        for g, v in self.geom_info.items():
            out[g] = dict(v)
        return out


# ----------------------------------------------------------------------------
# geometry objects, src/geometry.cpp (positions in doubled-grid units)
# ----------------------------------------------------------------------------
class _Box:
    def __init__(self, center, size, ab):
        self.lo = [min(center[d] - size[d] / 2, center[d] + size[d] / 2) for d in range(3)]
        self.hi = [max(center[d] - size[d] / 2, center[d] + size[d] / 2) for d in range(3)]
        self.ab = ab

    def inside(self, X, Y, Z):
        return ((X > self.lo[0]) & (X < self.hi[0]) & (Y > self.lo[1]) & (Y < self.hi[1])
                & (Z > self.lo[2]) & (Z < self.hi[2]))

    def bbox(self):
        return self.lo, self.hi

    def medium(self, X, Y, Z):
        return self.ab.epsilon, self.ab.mu, self.ab.e_amp, self.ab.m_amp


class _Sphere:
    def __init__(self, center, radius, ab):
        self.c = center
        self.r2 = radius * radius
        self.ab = ab

    def inside(self, X, Y, Z):
        dx = X - self.c[0]; dy = Y - self.c[1]; dz = Z - self.c[2]
        return dx * dx + dy * dy + dz * dz < self.r2

    def bbox(self):
        r = math.sqrt(self.r2)
        return [v - r for v in self.c], [v + r for v in self.c]

    def medium(self, X, Y, Z):
        return self.ab.epsilon, self.ab.mu, self.ab.e_amp, self.ab.m_amp


class _TwoMediumBox(_Box):
    """Two_Medium_Box, src/geometry.cpp:49-76"""

    def __init__(self, center, size, dim, m1, m2, rho):
        super().__init__(center, size, None)
        self.p1 = [center[d] - size[d] / 2 for d in range(3)]
        self.p2 = [center[d] + size[d] / 2 for d in range(3)]
        self.dim = dim
        self.m1, self.m2 = m1, m2
        self.rho = rho

    def val(self, X, Y, Z):
        p1, p2, dim = self.p1, self.p2, self.dim
        zq = (Z - p1[2]) / (p2[2] - p1[2]) * (dim[2] - 1)
        yq = (Y - p1[1]) / (p2[1] - p1[1]) * (dim[1] - 1)
        xq = (X - p1[0]) / (p2[0] - p1[0]) * (dim[0] - 1)
        return interp3(self.rho, (dim[2], dim[1], dim[0]), zq, yq, xq)

    def medium(self, X, Y, Z):
        v = self.val(X, Y, Z)
        eps = self.m1.epsilon * v + self.m2.epsilon * (1 - v)
        mu = self.m1.mu * v + self.m2.mu * (1 - v)
        ea = self.m1.e_amp[None, :] * v[:, None] + self.m2.e_amp[None, :] * (1 - v)[:, None]
        ma = self.m1.m_amp[None, :] * v[:, None] + self.m2.m_amp[None, :] * (1 - v)[:, None]
        return eps, mu, ea, ma


class _GeneralMediumBox(_TwoMediumBox):
    """General_Medium_Box, src/geometry.cpp:79-107"""

    def __init__(self, center, size, dim, rho, rho_fun, funs):
        super().__init__(center, size, dim, None, None, rho)
        self.rho_fun = rho_fun
        self.f_eps = np.array([f.epsilon for f in funs])
        self.f_mu = np.array([f.mu for f in funs])
        self.f_ea = np.stack([f.e_amp for f in funs]) if funs else np.zeros((0, 0))
        self.f_ma = np.stack([f.m_amp for f in funs]) if funs else np.zeros((0, 0))

    def medium(self, X, Y, Z):
        v = self.val(X, Y, Z)
        rf = self.rho_fun
        v = (v - rf[0]) / (rf[-1] - rf[0]) * (rf.size - 1)
        return (interp1_medium(self.f_eps, v), interp1_medium(self.f_mu, v),
                interp1_medium(self.f_ea, v), interp1_medium(self.f_ma, v))


def run_json(config: dict, datasets: Optional[Dict[str, np.ndarray]] = None, threads: int = 1) -> dict:
    """Set up, run to the config's stop condition and return the outputs."""
    sim = OracleSim(config, datasets, threads=threads)
    sim.run(config["stop condition"])
    return sim.outputs()
