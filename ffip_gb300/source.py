"""Source functions and sources with the interface of ffip/source.py."""
from __future__ import annotations

from copy import deepcopy

import numpy as np

from .geom import Vector3, cmp_shape


class Source_Function:
    @property
    def duration(self):
        return self.end_time - self.start_time


class Gaussian1(Source_Function):
    """First derivative of a Gaussian (source.py:31-53; the solver side is
    Gaussian1 in src/utility.cpp:260-264)."""

    def __init__(self, frequency, cutoff=4, start_time=0):
        self.frequency = float(frequency)
        self.cutoff = float(cutoff)
        self.start_time = float(start_time)
        self.width = 1 / (2 * np.pi * frequency)
        self.end_time = self.start_time + self.width * cutoff * 2
        self.offset_time = (self.start_time + self.end_time) / 2

    def get_json(self):
        return {"type": "Gaussian1", "frequency": self.frequency, "cutoff": self.cutoff, "start time": self.start_time}

    def __call__(self, t):
        arg = (t - self.offset_time) / self.width
        return arg * np.exp(-(arg ** 2) / 2)


class Gaussian2(Source_Function):
    """Second derivative of a Gaussian (src/utility.cpp:266-272)."""

    def __init__(self, frequency, cutoff=4, start_time=0):
        self.frequency = float(frequency)
        self.cutoff = float(cutoff)
        self.start_time = float(start_time)
        self.width = np.sqrt(2.0) / (2 * np.pi * frequency)
        self.end_time = self.start_time + self.width * cutoff * 2
        self.offset_time = (self.start_time + self.end_time) / 2

    def get_json(self):
        return {"type": "Gaussian2", "frequency": self.frequency, "cutoff": self.cutoff, "start time": self.start_time}

    def __call__(self, t):
        arg = ((t - self.offset_time) / self.width) ** 2
        return (1 - arg) * np.exp(-arg)


class Source:
    """Volume (or sheet, or point) current source, source.py:55-72."""

    def __init__(self, function, center=None, size=None, amplitude=1, field_component="Ex"):
        self.function = deepcopy(function)
        self.center = (center if center is not None else Vector3()).copy()
        self.size = (size if size is not None else Vector3()).copy()
        self.amplitude = float(amplitude)
        self.field_component = field_component

    def dump(self, datasets):
        pass

    def get_json(self):
        return {"type": "volume source", "center": self.center.get_json(), "size": self.size.get_json(),
                "amplitude": self.amplitude, "field component": self.field_component, "function": self.function.get_json()}


class Inhom_Source:
    """Source with a per-point complex amplitude on a grid: |a| scales the
    pulse, arg(a) shifts it in time (source.py:74-140; src/simulation.cpp:284-336)."""

    def __init__(self, function, amplitude=None, frequency=1, center=None, size=None, dim=None, field_component="Ex", suffix="0"):
        self.dim = (dim if dim is not None else Vector3()).round()
        self.function = deepcopy(function)
        self.frequency = float(frequency)
        self.center = (center if center is not None else Vector3()).copy()
        self.size = (size if size is not None else Vector3()).copy()
        self.field_component = field_component
        if callable(amplitude):
            self.amplitude = amplitude(np.stack(np.meshgrid(self.z, self.y, self.x, indexing="ij"), axis=-1))
        elif isinstance(amplitude, np.ndarray):
            self.amplitude = amplitude
        elif amplitude is None:
            self.amplitude = np.zeros(self.shape, dtype=complex)
        else:
            raise ValueError("amplitude input is not numpy array or a function")
        self.amplitude_dataset_name = "inhom source amplitude %s" % suffix
        self.phase_dataset_name = "inhom source phase %s" % suffix

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
    def shape(self):
        return (int(self.dim.z), int(self.dim.y), int(self.dim.x))

    @property
    def amplitude(self):
        return self._amp

    @amplitude.setter
    def amplitude(self, val):
        if not cmp_shape(self.shape, val.shape):
            raise ValueError("amplitude shape is not compatibale with source dimension")
        self._amp = np.array(val, copy=True)

    @property
    def numel(self):
        return int(self.dim.prod())

    def dump(self, datasets):
        datasets[self.amplitude_dataset_name] = np.abs(self.amplitude.ravel())
        datasets[self.phase_dataset_name] = np.angle(self.amplitude.ravel())

    def get_json(self):
        return {"type": "inhomogeneous source", "center": self.center.get_json(), "size": self.size.get_json(),
                "dimension": self.dim.get_json(), "field component": self.field_component,
                "amplitude dataset": self.amplitude_dataset_name, "phase dataset": self.phase_dataset_name,
                "frequency": self.frequency, "function": self.function.get_json()}
