"""Geometry, media and vectors with the interface of ffip/geom.py.

Every class builds the same config-JSON fragment as its namesake in the
reference (get_json) and the same input datasets (dump -> {name: array}
instead of writing into an HDF5 file).  Citations are to ffip/geom.py.
"""
from __future__ import annotations

import math
from copy import deepcopy
from numbers import Number

import numpy as np


def cmp_shape(shape1=(), shape2=()):
    """geom.py:12-20"""
    return len(shape1) == len(shape2) and all(a == b for a, b in zip(shape1, shape2))


def sph2cart(az, el, r):
    """geom.py:22-27"""
    rcos = r * np.cos(el)
    return rcos * np.cos(az), rcos * np.sin(az), r * np.sin(el)


def metadata_to_pts(*args):
    """meshgrid + stack of xn, ..., x1 (geom.py:29-31)"""
    return np.stack(np.meshgrid(*args, indexing="ij"), axis=-1)


class Vector3:
    """3-vector with the arithmetic of geom.py:33-170."""

    def __init__(self, x=0.0, y=0.0, z=0.0):
        self.x = float(x) if type(x) is int else x
        self.y = float(y) if type(y) is int else y
        self.z = float(z) if type(z) is int else z

    def _other(self, o):
        return Vector3(o, o, o) if isinstance(o, Number) else o

    def __eq__(self, o):
        return self.x == o.x and self.y == o.y and self.z == o.z

    def __add__(self, o):
        o = self._other(o)
        return Vector3(self.x + o.x, self.y + o.y, self.z + o.z)

    def __sub__(self, o):
        o = self._other(o)
        return Vector3(self.x - o.x, self.y - o.y, self.z - o.z)

    def __mul__(self, o):
        if type(o) is Vector3:
            return self.dot(o)
        if isinstance(o, Number):
            return self.scale(o)
        raise TypeError("No operation known for 'Vector3 * {}'".format(type(o)))

    def __rmul__(self, o):
        if isinstance(o, Number):
            return self.scale(o)
        raise TypeError("No operation known for '{} * Vector3'".format(type(o)))

    def __truediv__(self, o):
        if type(o) is Vector3:
            return Vector3(self.x / o.x, self.y / o.y, self.z / o.z)
        if isinstance(o, Number):
            return Vector3(self.x / o, self.y / o, self.z / o)
        raise TypeError("No operation known for 'Vector3 / {}'".format(type(o)))

    def __getitem__(self, i):
        if i in (0, 1, 2):
            return (self.x, self.y, self.z)[i]
        raise IndexError("No value at index {}".format(i))

    def __setitem__(self, i, v):
        if i == 0:
            self.x = v
        elif i == 1:
            self.y = v
        elif i == 2:
            self.z = v
        else:
            raise IndexError("No value at index {}".format(i))

    def __repr__(self):
        return "Vector3<{}, {}, {}>".format(self.x, self.y, self.z)

    def __array__(self, dtype=None, copy=None):
        return np.array([self.x, self.y, self.z], dtype=dtype)

    def conj(self):
        return Vector3(self.x.conjugate(), self.y.conjugate(), self.z.conjugate())

    def scale(self, s):
        return Vector3(self.x * s, self.y * s, self.z * s)

    def dot(self, v):
        return self.x * v.x + self.y * v.y + self.z * v.z

    def cdot(self, v):
        return self.conj().dot(v)

    def cross(self, v):
        return Vector3(self.y * v.z - self.z * v.y, self.z * v.x - self.x * v.z, self.x * v.y - self.y * v.x)

    def norm(self):
        return math.sqrt(abs(self.dot(self)))

    def unit(self):
        return self.scale(1 / self.norm())

    def prod(self):
        return self.x * self.y * self.z

    def close(self, v, tol=1.0e-7):
        return abs(self.x - v.x) <= tol and abs(self.y - v.y) <= tol and abs(self.z - v.z) <= tol

    def rotate(self, axis, theta):
        u = axis.unit()
        vpar = u.scale(u.dot(self))
        return vpar + ((self - vpar).scale(math.cos(theta)) + u.cross(self).scale(math.sin(theta)))

    def get_json(self):
        return [self.x, self.y, self.z]

    def ceil(self):
        return Vector3(math.ceil(self.x), math.ceil(self.y), math.ceil(self.z))

    def floor(self):
        return Vector3(math.floor(self.x), math.floor(self.y), math.floor(self.z))

    def round(self):
        return Vector3(round(self.x), round(self.y), round(self.z))

    def copy(self):
        return Vector3(self.x, self.y, self.z)


class Susceptibility:
    """sigma * (a0 + a1 jw) / (b0 + b1 jw - b2 w^2), geom.py:229-260"""

    def __init__(self, sigma=1.0):
        self.sigma = sigma

    def build_eqs(self, a0=0.0, a1=0.0, b0=0.0, b1=0.0, b2=0.0):
        self.a0, self.a1, self.b0, self.b1, self.b2 = (float(v) for v in (a0, a1, b0, b1, b2))

    def __eq__(self, o):
        return (self.a0, self.a1, self.b0, self.b1, self.b2) == (o.a0, o.a1, o.b0, o.b1, o.b2)

    def get_epsilon(self, frequency):
        w = 2 * np.pi * frequency
        return self.sigma * (self.a0 + self.a1 * 1j * w) / (self.b0 + 1j * w * self.b1 - w * w * self.b2)

    def get_dis_epsilon(self, frequency, dt):
        """The susceptibility the discrete ADE update realises at a frequency."""
        c0 = 2 * self.b2 + self.b1 * dt
        c1 = (4 * self.b2 - 2 * self.b0 * dt * dt) / c0
        c2 = (-2 * self.b2 + self.b1 * dt) / c0
        c3 = (2 * self.a0 * dt * dt) / c0
        z = np.exp(1j * 2 * np.pi * frequency * dt)
        return self.sigma * c3 * z / (z ** 2 - c1 * z - c2)


class LorentzianSusceptibility(Susceptibility):
    def __init__(self, frequency=0.0, gamma=0.0, **kwargs):
        super().__init__(**kwargs)
        w, g = 2 * np.pi * frequency, 2 * np.pi * gamma
        self.build_eqs(a0=w ** 2, b0=w ** 2, b1=g, b2=1)
        self.frequency, self.gamma = float(frequency), float(gamma)

    def get_json(self):
        return {"type": "Lorentz", "frequency": self.frequency, "gamma": self.gamma, "amplitude": self.sigma}


class DrudeSusceptibility(Susceptibility):
    def __init__(self, frequency=0.0, gamma=0.0, **kwargs):
        super().__init__(**kwargs)
        w, g = 2 * np.pi * frequency, 2 * np.pi * gamma
        self.build_eqs(a0=w ** 2, b1=g, b2=1)
        self.frequency, self.gamma = float(frequency), float(gamma)

    def get_json(self):
        return {"type": "Drude", "frequency": self.frequency, "gamma": self.gamma, "amplitude": self.sigma}


class DeybeSusceptibility(Susceptibility):
    def __init__(self, tau=0.0, **kwargs):
        super().__init__(**kwargs)
        self.build_eqs(a0=1, b0=1, b1=tau)
        self.tau = float(tau)

    def get_json(self):
        return {"type": "Deybe", "tau": self.tau, "amplitude": self.sigma}


class Medium:
    """geom.py:173-227"""

    def __init__(self, epsilon=1, mu=1, E_conductivity=0, M_conductivity=0, E_susceptibilities=(), M_susceptibilities=()):
        self.epsilon = float(epsilon)
        self.mu = float(mu)
        self.E_susceptibilities = deepcopy(list(E_susceptibilities))
        self.M_susceptibilities = deepcopy(list(M_susceptibilities))
        self.E_conductivity = float(E_conductivity)
        self.M_conductivity = float(M_conductivity)

    def get_imp(self):
        return math.sqrt(self.mu / self.epsilon)

    def get_c(self):
        return 1 / math.sqrt(self.mu * self.epsilon)

    def get_json(self):
        return {"epsilon": self.epsilon, "mu": self.mu, "electric conductivity": self.E_conductivity,
                "magnetic conductivity": self.M_conductivity,
                "electric susceptibility": [s.get_json() for s in self.E_susceptibilities],
                "magnetic susceptibility": [s.get_json() for s in self.M_susceptibilities]}

    def get_epsilon(self, frequency):
        res = self.epsilon - 1j * self.E_conductivity / (2 * np.pi * frequency)
        for s in self.E_susceptibilities:
            res += s.get_epsilon(frequency)
        return res

    def get_dis_epsilon(self, frequency, dt):
        z = np.exp(1j * 2 * np.pi * frequency * dt)
        res = self.epsilon + 2 * dt * z / (z ** 2 - 1) * self.E_conductivity
        for s in self.E_susceptibilities:
            res += s.get_dis_epsilon(frequency, dt)
        return res


class GeometricObject:
    def __init__(self, material=None, center=None):
        self.material = deepcopy(material if material is not None else Medium())
        self.center = (center if center is not None else Vector3()).copy()

    def shift(self, vec):
        c = deepcopy(self)
        c.center += vec
        return c

    def dump(self, datasets):
        pass


class Sphere(GeometricObject):
    def __init__(self, radius, **kwargs):
        self.radius = radius
        super().__init__(**kwargs)

    @property
    def radius(self):
        return self._radius

    @radius.setter
    def radius(self, v):
        self._radius = float(v) if v > 0 else 0.0

    def get_json(self):
        return {"type": "sphere", "center": self.center.get_json(), "radius": self.radius, "medium": self.material.get_json()}


class Box(GeometricObject):
    def __init__(self, size=None, **kwargs):
        self.size = size if size is not None else Vector3()
        super().__init__(**kwargs)

    @property
    def size(self):
        return self._size

    @size.setter
    def size(self, v):
        self._size = v.copy() if (v.x > 0 and v.y > 0 and v.z > 0) else Vector3()

    def get_json(self):
        return {"type": "box", "center": self.center.get_json(), "size": self.size.get_json(), "medium": self.material.get_json()}


class _DensityBox:
    """Shared grid logic of the density boxes (geom.py:375-430, 493-526)."""

    def _init_density(self, density):
        if callable(density):
            self.density = density(np.stack(np.meshgrid(self.z, self.y, self.x, indexing="ij"), axis=-1))
        elif isinstance(density, np.ndarray):
            self.density = density
        elif density is None:
            self.density = np.zeros(self.shape, dtype=float)
        else:
            raise ValueError("amplitude input is not numpy array or a function")

    @property
    def density(self):
        return self._density

    @density.setter
    def density(self, val):
        if not cmp_shape(self.shape, val.shape):
            raise ValueError("density size is not compatible with the box dimension")
        self._density = np.array(val, copy=True)

    @property
    def x(self):
        return np.linspace(self.center.x - self.size.x / 2, self.center.x + self.size.x / 2, int(self.dim.x))

    @property
    def y(self):
        return np.linspace(self.center.y - self.size.y / 2, self.center.y + self.size.y / 2, int(self.dim.y))

    @property
    def z(self):
        return np.linspace(self.center.z - self.size.z / 2, self.center.z + self.size.z / 2, int(self.dim.z))

    @property
    def dimension(self):
        return self.dim

    @property
    def shape(self):
        return (int(self.dim.z), int(self.dim.y), int(self.dim.x))

    @property
    def numel(self):
        return int(self.dim.prod())


class Two_Medium_Box(_DensityBox):
    """epsilon = medium1 * rho + medium2 * (1 - rho), rho trilinear on a grid
    (geom.py:375-443; the solver side is src/geometry.cpp:49-76)."""

    def __init__(self, size=None, center=None, dim=None, density=None, medium1=None, medium2=None, suffix="0"):
        self.size = (size if size is not None else Vector3()).copy()
        self.center = (center if center is not None else Vector3()).copy()
        self.dim = (dim if dim is not None else Vector3()).round()
        self.medium1 = deepcopy(medium1 if medium1 is not None else Medium())
        self.medium2 = deepcopy(medium2 if medium2 is not None else Medium())
        self._init_density(density)
        self.dataset_name = "two medium box %s" % suffix

    def dump(self, datasets):
        datasets[self.dataset_name] = self.density.ravel()

    def get_json(self):
        return {"type": "two medium box", "center": self.center.get_json(), "size": self.size.get_json(),
                "dimension": self.dim.get_json(), "density dataset": self.dataset_name,
                "medium1": self.medium1.get_json(), "medium2": self.medium2.get_json()}


class General_Medium_Box(_DensityBox):
    """Two-pole medium whose pole amplitudes follow epsilon_fun(rho) at one
    frequency (geom.py:446-559)."""

    def __init__(self, size=None, center=None, dim=None, frequency=1.0, density=None, epsilon_fun=None, e_sus=(), suffix="0"):
        self.size = (size if size is not None else Vector3()).copy()
        self.center = (center if center is not None else Vector3()).copy()
        self.dim = (dim if dim is not None else Vector3()).round()
        self.frequency = float(frequency)
        if len(e_sus) != 2:
            raise ValueError("Currently only support two poles")
        self.e_sus = deepcopy(list(e_sus))
        self.medium = Medium(epsilon=1, E_susceptibilities=self.e_sus)
        self.epsilon_fun = deepcopy(epsilon_fun)
        self.e1 = self.e_sus[0].get_epsilon(frequency) / self.e_sus[0].sigma
        self.e2 = self.e_sus[1].get_epsilon(frequency) / self.e_sus[1].sigma
        self.mat = np.array([[np.real(self.e1), np.real(self.e2)], [np.imag(self.e1), np.imag(self.e2)]])
        self.invmat = np.linalg.inv(self.mat)
        self._init_density(density)
        prefix = "general medium box %s " % suffix
        self.density_dataset = prefix + "density"
        self.density_fun_dataset = prefix + "density function"
        self.epsilon_dataset = prefix + "epsilon"
        self.mu_dataset = prefix + "mu"
        self.e_sus_amp_dataset = prefix + "e sus amp"
        self.m_sus_amp_dataset = prefix + "m sus amp"

    def dump(self, datasets):
        rho = np.linspace(0, 1, 1000)
        eps = self.epsilon_fun(rho)
        amp = np.transpose(self.invmat @ np.stack((np.real(eps) - 1, np.imag(eps)), axis=0))
        datasets[self.density_dataset] = self.density.ravel()
        datasets[self.density_fun_dataset] = rho.ravel()
        datasets[self.epsilon_dataset] = np.ones(rho.size)
        datasets[self.mu_dataset] = np.ones(rho.size)
        datasets[self.e_sus_amp_dataset] = amp.flatten()
        datasets[self.m_sus_amp_dataset] = np.ones(0)

    def get_json(self):
        return {"type": "general medium box", "center": self.center.get_json(), "size": self.size.get_json(),
                "dimension": self.dim.get_json(), "density dataset": self.density_dataset,
                "density function dataset": self.density_fun_dataset, "epsilon dataset": self.epsilon_dataset,
                "mu dataset": self.mu_dataset, "electric susceptibility amplitudes dataset": self.e_sus_amp_dataset,
                "magnetic susceptibility amplitudes dataset": self.m_sus_amp_dataset, "medium": self.medium.get_json()}


def planar_polygon(polygon, center=None, height=np.inf):
    """Density function of an extruded planar polygon (ffip/geom.py:569-590):
    returns f(req_pts) with req_pts[..., (z, y, x)] giving 1 where (x, y) -
    center lies strictly inside the polygon (check_inside on the GPU) and
    |z - center.z| < height / 2, else 0.  `polygon` is a shapely-like object
    (`.exterior` coordinates, or `.geoms` of several) or an (m, 2) vertex
    array; several polygons are OR-ed."""
    from .native import check_inside
    center = center if center is not None else Vector3()

    def rings(g):
        if hasattr(g, "geoms"):
            for h in g.geoms:
                yield from rings(h)
        elif hasattr(g, "exterior"):
            yield np.asarray(g.exterior.coords if hasattr(g.exterior, "coords") else g.exterior, dtype=np.float64)
        else:
            yield np.asarray(g, dtype=np.float64)

    def internal(req_pts):
        req_pts = np.asarray(req_pts, dtype=np.float64)
        xy = np.stack((req_pts[..., 2] - center.x, req_pts[..., 1] - center.y), axis=-1)
        z_check = np.abs(req_pts[..., 0] - center.z) < (height / 2)
        res = np.zeros(req_pts.shape[:-1], dtype=bool)
        for ring in rings(polygon):
            res |= check_inside(req_pts=xy, poly_pts=ring) & z_check
        return res * 1

    return internal


def getgrid(center=None, size=None, dim=None):
    center = center if center is not None else Vector3()
    size = size if size is not None else Vector3()
    dim = dim if dim is not None else Vector3()
    return (np.linspace(center.z - size.z / 2, center.z + size.z / 2, int(dim.z)),
            np.linspace(center.y - size.y / 2, center.y + size.y / 2, int(dim.y)),
            np.linspace(center.x - size.x / 2, center.x + size.x / 2, int(dim.x)))
