"""Simulation front-end with the interface of ffip/simulation.py.

`Simulation(...).run(stop_condition)` builds the same config JSON as the
reference (get_json, simulation.py:362-402) and the same input datasets, but
instead of writing config.json + input.h5 and launching
`mpirun -np N run_sim_json` (simulation.py:404-431) it runs the GB300 stepper
in-process through the C ABI and fills the DFT / geometry-info objects from
the returned datasets.  The adjoint helpers (Adjoint_Source, Adjoint_Flux,
Adjoint_Volume) follow simulation.py:544-915; the sensitivity correlation and
its transposed interpolation run on the GPU (ffip_sensitivity).

Rebuild-only keyword arguments of Simulation: precision ("fp64" | "fp32"),
engine ("auto" | "fused" | "unfused"), device (CUDA index).
"""
from __future__ import annotations

import ctypes
import json
from copy import copy, deepcopy
from math import pi

import numpy as np
from scipy.interpolate import RegularGridInterpolator

from . import native
from .geom import General_Medium_Box, Medium, Two_Medium_Box, Vector3, cmp_shape
from .source import Inhom_Source

direction_dict = {"x": 0, "y": 1, "z": 2}
side_dict = {"positive": 1, "negative": -1}


class Fields_DFT:
    """One DFT volume monitor (simulation.py:17-91)."""

    def __init__(self, center, size, frequency, field_component, suffix="0", degenerate=False, dx=0):
        self.suffix = str(suffix)
        self.group_name = "volume fields dft %s" % suffix
        self.center = center.copy()
        self.size = size.copy()
        self.degenerate = bool(degenerate)
        self.dx = float(dx)
        if not self.degenerate and dx == 0:
            raise ValueError("for non degenerate dft, dx must be provided")
        self.frequency = np.sort(np.asarray(frequency, dtype=float))
        self.frequency_config = self.frequency.tolist()
        self.field_component = field_component

    def get_json(self):
        return {"type": "volume fields dft", "center": self.center.get_json(), "size": self.size.get_json(),
                "frequency": self.frequency_config, "field component": self.field_component, "output group": self.group_name}

    @property
    def values(self):
        return self.v

    def read(self, outputs):
        g = outputs[self.group_name]
        self.frequency = np.asarray(g["f"])
        self.x, self.y, self.z = np.asarray(g["x"]), np.asarray(g["y"]), np.asarray(g["z"])
        self.v = g["real"] + 1j * g["imag"]
        # the output grid as written (before the widening below)
        self.raw = (self.frequency.copy(), self.z.copy(), self.y.copy(), self.x.copy(), self.v)
        if not self.degenerate:
            # size-1 axes are widened so that interpolation works (simulation.py:55-72)
            if self.frequency.size == 1:
                self.frequency = self.frequency * np.array([0.9, 1.1])
            if self.x.size == 1:
                self.x = self.x + np.array([-self.dx / 2, self.dx / 2])
            if self.y.size == 1:
                self.y = self.y + np.array([-self.dx / 2, self.dx / 2])
            if self.z.size == 1:
                self.z = self.z + np.array([-self.dx / 2, self.dx / 2])
            for i in range(4):
                if self.v.shape[i] == 1:
                    self.v = np.concatenate((self.v, self.v), axis=i)

    def __call__(self, f, z, y, x, substract=None, **kwargs):
        interp = self.get_interpolant(substract, **kwargs)
        return interp(np.stack(np.meshgrid(f, z, y, x, indexing="ij"), axis=-1))

    def get_interpolant(self, substract=None, **kwargs):
        if substract is not None and not isinstance(substract, Fields_DFT):
            raise TypeError("Substract is not an instance of Fields_DFT")
        vals = self.values - substract.values if substract is not None else self.values
        return RegularGridInterpolator((self.frequency, self.z, self.y, self.x), vals, **kwargs)

    def get_metadata(self):
        return self.frequency, self.z, self.y, self.x


class Flux_Region:
    """Poynting flux through a plane from E1 and H2 monitors (simulation.py:94-210)."""

    def __init__(self, sim, center, size, frequency, weight):
        dim = (size.x != 0) + (size.y != 0) + (size.z != 0)
        if dim != 2:
            raise NameError("Flux region dimension %d is invalid" % dim)
        self.direction = 0 if size.x == 0 else 1 if size.y == 0 else 2
        self.weight = np.array(weight, copy=True)
        self.center, self.size = center.copy(), size.copy()
        self.frequency = np.sort(np.asarray(frequency))
        self.dx = sim.dx
        self._sim = sim
        self._e1_dft = sim.add_dft_fields(center=center, size=size, frequency=frequency, field_component=self.e1_str)
        self._h2_dft = sim.add_dft_fields(center=center, size=size, frequency=frequency, field_component=self.h2_str)

    @property
    def e1_str(self):
        return "E" + "xyz"[(self.direction + 1) % 3]

    @property
    def h2_str(self):
        return "H" + "xyz"[(self.direction + 2) % 3]

    @property
    def e1_dft(self):
        return self._e1_dft

    @property
    def h2_dft(self):
        return self._h2_dft

    def get_fields(self, scale=1, substract=None, **kwargs):
        if substract is not None and not isinstance(substract, Flux_Region):
            raise TypeError("Substract is not an instance of Flux_Region")
        e1i = self.e1_dft.get_interpolant(substract=substract.e1_dft if substract is not None else None, **kwargs)
        h2i = self.h2_dft.get_interpolant(substract=substract.h2_dft if substract is not None else None, **kwargs)
        pts = self.get_pts(scale=scale)
        return e1i(pts), h2i(pts)

    def get_len(self, scale=1):
        return (self.size / self.dx * scale).round() + Vector3(1, 1, 1)

    def get_metadata(self, scale=1):
        n = self.get_len(scale=scale)
        p1, p2 = self.center - self.size / 2, self.center + self.size / 2
        return (self.frequency, np.linspace(p1.z, p2.z, int(n.z)), np.linspace(p1.y, p2.y, int(n.y)),
                np.linspace(p1.x, p2.x, int(n.x)))

    def get_pts(self, scale=1):
        return np.stack(np.meshgrid(*self.get_metadata(scale=scale), indexing="ij"), axis=-1)

    def get_int_weights(self, scale=1):
        n = self.get_len(scale=scale)
        x, y, z = np.ones(int(n.x)), np.ones(int(n.y)), np.ones(int(n.z))
        meas = 1
        for ln, sz in ((n.x, self.size.x), (n.y, self.size.y), (n.z, self.size.z)):
            if ln > 1:
                meas *= sz / (ln - 1)
        for item in (x, y, z):
            if item.size > 1:
                item[0] = item[-1] = 0.5
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        return X * Y * Z * meas * self.weight

    def get_values(self, scale=1, substract=None, device=False, **kwargs):
        """Flux per frequency.  device=True (rebuild-only): the same sum on the
        GPU from the monitors of a simulation kept there (run(keep=True)),
        without copying them back (ffip_flux)."""
        if device:
            if substract is not None or kwargs:
                raise ValueError("the device flux takes neither substract nor interpolation options")
            kept = getattr(self._sim, "_kept", None)
            if kept is None:
                raise RuntimeError("the device flux needs a simulation kept on the device (run(keep=True))")
            f, z, y, x = self.get_metadata(scale=scale)
            return kept["sim"].flux(self.e1_dft.group_name, self.h2_dft.group_name, x, y, z, self.get_int_weights(scale=scale),
                                    self.frequency)
        e1, h2 = self.get_fields(scale=scale, substract=substract, **kwargs)
        flux = np.real(e1 * np.conj(h2)) * self.get_int_weights(scale=scale)
        return np.sum(flux, axis=(1, 2, 3))

    def get_interpolant(self, scale=1, substract=None):
        return RegularGridInterpolator((self.frequency,), self.get_values(scale=scale, substract=substract))


class Flux_Box:
    """Six flux planes of a box, outward weights (simulation.py:212-250)."""

    def __init__(self, sim, center, size, frequency):
        self._flux_regions = []
        self.frequency = np.sort(np.asarray(frequency))
        for d in range(3):
            for side in (-1, 1):
                p1, p2 = center - size / 2, center + size / 2
                if side == -1:
                    p2[d] = p1[d]
                else:
                    p1[d] = p2[d]
                self._flux_regions.append(sim.add_flux_region(center=(p1 + p2) / 2, size=p2 - p1, frequency=frequency, weight=side))

    @property
    def flux_regions(self):
        return self._flux_regions

    def get_flux_region(self, direction="x", side="negative"):
        return self.flux_regions[direction_dict[direction] * 2 + (0 if side_dict[side] == -1 else 1)]

    def get_values(self, scale=1, substract=None, device=False, **kwargs):
        if substract is not None and not isinstance(substract, Flux_Box):
            raise TypeError("Substract is not an instance of Flux_Box")
        return sum(r.get_values(scale=scale, substract=substract.flux_regions[i] if substract is not None else None,
                                device=device, **kwargs)
                   for i, r in enumerate(self.flux_regions))

    def get_interpolant(self, scale=1, substract=None, **kwargs):
        return RegularGridInterpolator((self.frequency,), self.get_values(scale=scale, substract=substract, **kwargs))


class Geom_Info:
    """Coordinates of one component's grid points inside a geometry
    (simulation.py:253-283; written by src/simulation.cpp:190-233, where the
    coordinates pass through a std::vector<int>)."""

    def __init__(self, index=0, field_component="Ex"):
        self.field_component = str(field_component)
        self.index = int(index)
        self.gname = "geometry info request %d %s" % (self.index, self.field_component)

    def read(self, outputs):
        g = outputs[self.gname]
        self._x, self._y, self._z = (np.asarray(g[k]) for k in ("x", "y", "z"))

    def get_json(self):
        return {"field component": self.field_component, "geometry index": self.index, "output group": self.gname}

    @property
    def x(self):
        return self._x

    @property
    def y(self):
        return self._y

    @property
    def z(self):
        return self._z


class Symmetry:
    def __init__(self, direction="x", phase_factor=1):
        self.direction = direction
        self.phase_factor = int(phase_factor)

    def get_json(self):
        return {"direction": self.direction, "phase factor": self.phase_factor}


class run_until_time:
    def __init__(self, time=0):
        self.time = float(time)

    def get_json(self):
        return {"type": "time", "time": self.time}


class run_until_dft:
    def __init__(self, center=None, size=None, frequency=1, field_component="Ex", time_interval_examined=1, var=1e-2):
        self.center = (center if center is not None else Vector3()).copy()
        self.size = (size if size is not None else Vector3()).copy()
        self.field_component = str(field_component)
        self.time_interval_examined = float(time_interval_examined)
        self.var = float(var)
        self.frequency = float(frequency)

    def get_json(self):
        return {"type": "dft", "center": self.center.get_json(), "size": self.size.get_json(),
                "field component": self.field_component, "time interval examined": self.time_interval_examined,
                "variation": self.var, "frequency": self.frequency}


class run_until_fields_decay:
    def __init__(self, position=None, field_component="Ez", time_interval_examined=1, decayed_by=1e-3):
        self.position = (position if position is not None else Vector3()).copy()
        self.field_component = str(field_component)
        self.time_interval_examined = float(time_interval_examined)
        self.decayed_by = float(decayed_by)

    def get_json(self):
        return {"type": "decay", "position": self.position.get_json(), "field component": self.field_component,
                "time interval examined": self.time_interval_examined, "decayed by": self.decayed_by}


class PML:
    """CPML layer (simulation.py:519-542).  sigma_max=None takes the default
    0.8 (order + 1) / dx at Simulation construction; an explicit sigma_max is
    kept (the reference's PML.__init__ discards it, simulation.py:526)."""

    def __init__(self, thickness, direction=None, side=None, k_max=1, order=3, sigma_max=None):
        self.thickness = float(thickness)
        self.direction = direction
        self.side = side
        self.k_max = float(k_max)
        self.order = int(order)
        self.sigma_max = sigma_max

    def get_json(self):
        res = {"thickness": self.thickness}
        if self.direction is not None:
            res["direction"] = self.direction
        if self.side is not None:
            res["side"] = self.side
        res["k max"] = self.k_max if self.k_max is not None else 1.0
        res["order"] = self.order if self.order is not None else 3
        res["sigma max"] = self.sigma_max
        return res


class Simulation:
    """simulation.py:286-464, run in-process on the GPU."""

    def __init__(self, size, resolution, pmls=(), geometry=(), sources=(), symmetry=(), default_material=None,
                 periodic=False, progress_interval=4, courant=0.5, input_file="empty.h5", fields_output_file="output.h5",
                 precision="fp64", engine="auto", device=None):
        self.size = size.copy()
        self.resolution = float(resolution)
        self.geometry = deepcopy(list(geometry))
        self.sources = deepcopy(list(sources))
        self.symmetry = deepcopy(list(symmetry))
        self.default_material = deepcopy(default_material if default_material is not None else Medium())
        self.periodic = deepcopy(periodic)
        self.progress_interval = float(progress_interval)
        self.courant = float(courant)
        self.pmls = deepcopy(list(pmls))
        self.input_file = copy(input_file)
        self.fields_output_file = copy(fields_output_file)
        self.precision, self.engine, self.device = precision, engine, device
        self.dft_fields, self.flux_regions, self.flux_boxes, self.geom_info_requests = [], [], [], []
        self.outputs = None
        for p in self.pmls:
            if p.sigma_max is None:
                p.sigma_max = 0.8 * (1 + p.order) * resolution

    @property
    def dx(self):
        return 1 / self.resolution

    def dump(self, datasets=None):
        """Input datasets ({name: array}) that the reference writes to input.h5."""
        datasets = {} if datasets is None else datasets
        for g in self.geometry:
            if hasattr(g, "dump"):
                g.dump(datasets)
        for s in self.sources:
            s.dump(datasets)
        return datasets

    def get_json(self, stop_condition, decomposition=None):
        res = {"courant number": self.courant, "resolution": self.resolution, "size": self.size.get_json(),
               "default material": self.default_material.get_json(), "progress interval": self.progress_interval,
               "input file": self.input_file, "fields output file": self.fields_output_file,
               "stop condition": stop_condition.get_json()}
        if decomposition is not None:
            res["decomposition"] = decomposition
        if self.symmetry:
            # the reference serialises self.periodic here (simulation.py:380)
            res["symmetry"] = [s.get_json() for s in self.symmetry]
        if self.pmls:
            res["PML"] = [p.get_json() for p in self.pmls]
        if self.periodic:
            res["periodic"] = self.periodic
        if self.geometry:
            res["geometry"] = [g.get_json() for g in self.geometry]
        if self.sources:
            res["sources"] = [s.get_json() for s in self.sources]
        if self.dft_fields:
            res["fields output"] = [d.get_json() for d in self.dft_fields]
        if self.geom_info_requests:
            res["geometry info request"] = [g.get_json() for g in self.geom_info_requests]
        return res

    def config(self, stop_condition):
        cfg = self.get_json(stop_condition)
        cfg["precision"] = self.precision
        cfg["engine"] = self.engine
        if self.device is not None:
            cfg["device"] = int(self.device)
        return cfg

    def run(self, stop_condition, decomposition=None, np=1, skip=False, pop=False, write_config=None, keep=False,
            **kwargs):
        """Runs to the stop condition and reads the outputs back.  `decomposition`
        and `np` (MPI ranks of the reference) are accepted and ignored: one GPU
        runs the whole domain.  write_config: optional path to also write the
        config JSON (what the reference's run_sim_json would read).

        keep=True keeps the device simulation between runs: when the config is
        unchanged and only two-medium-box densities or inhomogeneous-source
        amplitude/phase datasets differ, the next run updates them in place
        (ffip_set_density / ffip_set_source_data) instead of building the
        simulation again, which is what a design loop repeats."""
        cfg = self.config(stop_condition)
        if write_config:
            with open(write_config, "w") as f:
                json.dump(self.get_json(stop_condition, decomposition), f, indent=4)
        if not skip:
            datasets = self.dump()
            if keep:
                self.outputs = self._run_kept(cfg, datasets)
            else:
                self.release()
                self.outputs = native.run_json(cfg, datasets)
        for item in self.dft_fields:
            item.read(self.outputs)
        for item in self.geom_info_requests:
            item.read(self.outputs)

    def _run_kept(self, cfg, datasets):
        kept = getattr(self, "_kept", None)
        if kept is not None and kept["cfg"] == cfg and kept["names"] == set(datasets):
            density = {g.dataset_name for g in self.geometry if isinstance(g, Two_Medium_Box)}
            source = set()
            for src in self.sources:
                if isinstance(src, Inhom_Source):
                    source |= {src.amplitude_dataset_name, src.phase_dataset_name}
            changed = [k for k, v in datasets.items() if not np.array_equal(kept["data"][k], v)]
            if all(k in density or k in source for k in changed):
                sim = kept["sim"]
                for k in changed:
                    if k in density:
                        sim.set_density(k, datasets[k])
                src_changed = {k: datasets[k] for k in changed if k in source}
                if src_changed:
                    sim.set_source_data(src_changed)
                if not changed:
                    sim.reset()
                for k in changed:
                    kept["data"][k] = np.array(datasets[k], copy=True)
                sim.run(cfg["stop condition"])
                return sim.outputs()
        self.release()
        sim = native.NativeSim(cfg, datasets)
        self._kept = {"cfg": cfg, "names": set(datasets), "sim": sim,
                      "data": {k: np.array(v, copy=True) for k, v in datasets.items()}}
        sim.run(cfg["stop condition"])
        return sim.outputs()

    def release(self):
        """Frees a simulation kept on the device by run(keep=True)."""
        kept = getattr(self, "_kept", None)
        if kept is not None:
            kept["sim"].close()
            self._kept = None

    def add_geometry(self, geom):
        self.geometry.insert(0, geom)

    def add_source(self, src):
        self.sources.insert(0, src)

    def request_geom_info(self, geom, field_component="Ex"):
        for i, g in enumerate(self.geometry):
            if g is geom:
                req = Geom_Info(index=i, field_component=field_component)
                self.geom_info_requests.append(req)
                return req
        raise ValueError("Geometry non-existed")

    def add_dft_fields(self, center=None, size=None, frequency=(), field_component="Ex"):
        res = Fields_DFT(center if center is not None else Vector3(), size if size is not None else Vector3(), frequency,
                         field_component, str(len(self.dft_fields)), degenerate=False, dx=self.dx)
        self.dft_fields.append(res)
        return res

    def add_flux_region(self, center=None, size=None, frequency=(), weight=1):
        res = Flux_Region(self, center=center if center is not None else Vector3(), size=size if size is not None else Vector3(),
                          frequency=frequency, weight=weight)
        self.flux_regions.append(res)
        return res

    def add_flux_box(self, center=None, size=None, frequency=()):
        res = Flux_Box(self, center=center if center is not None else Vector3(), size=size if size is not None else Vector3(),
                       frequency=frequency)
        self.flux_boxes.append(res)
        return res


def field_match_objective(obj_val, component="Ex", weight=1):
    """(components, d/dE* of F, F) triplets (simulation.py:544-582)."""
    if component in ("Ex", "Ey", "Ez"):
        def fun1(val):
            return np.sum(0.5 * np.ravel(weight) * np.abs(val.ravel() - obj_val.ravel()) ** 2)

        def fpconj1(val):
            return (np.conj(val - obj_val) * weight,)
        return [component], fpconj1, fun1
    if component in ("|Ex|", "|Ey|", "|Ez|"):
        def fun2(val):
            return np.sum(0.5 * np.ravel(weight) * (np.abs(val).ravel() - obj_val.ravel()) ** 2)

        def fpconj2(val):
            return ((1 - obj_val / np.abs(val)) * np.conj(val) * weight,)
        return [component[1:-1]], fpconj2, fun2
    if component == "|E|":
        def fun3(ex, ey, ez):
            val = np.sqrt(np.abs(ex) ** 2 + np.abs(ey) ** 2 + np.abs(ez) ** 2)
            return np.sum(0.5 * (np.ravel(val) - np.ravel(obj_val)) ** 2 * np.ravel(weight))

        def fpconj3(ex, ey, ez):
            val = np.sqrt(np.abs(ex) ** 2 + np.abs(ey) ** 2 + np.abs(ez) ** 2)
            return tuple((1 - obj_val / val) * np.conj(e) * weight for e in (ex, ey, ez))
        return ["Ex", "Ey", "Ez"], fpconj3, fun3
    raise ValueError("unknown objective component " + str(component))


class Adjoint_Source:
    """Adjoint sources from objective derivatives at monitor points
    (simulation.py:648-757): the adjoint source amplitude is dF/dE* there."""

    def __init__(self, adjoint_simulation, forward_simulation, function, frequency=1.0, center=None, size=None, dim=None,
                 functionals=(), udfs=()):
        self.adjoint_simulation = adjoint_simulation
        self.forward_simulation = forward_simulation
        self.frequency = float(frequency)
        self.center = (center if center is not None else Vector3()).copy()
        self.size = (size if size is not None else Vector3()).copy()
        dim = dim if dim is not None else Vector3()
        self.dim = dim.round()
        self.functionals = deepcopy(list(functionals))
        self.udfs = list(udfs)
        self.function = deepcopy(function)
        self.forward_dfts, self.adjoint_sources, self.forward_fields = {}, {}, {}
        p1 = self.center - self.size / 2
        self.x = np.linspace(p1.x, p1.x + self.size.x, int(dim.x))
        self.y = np.linspace(p1.y, p1.y + self.size.y, int(dim.y))
        self.z = np.linspace(p1.z, p1.z + self.size.z, int(dim.z))
        for func in self.functionals:
            if not cmp_shape(self.shape, func[1].shape):
                raise ValueError("objective values does not match the shape")
            self.udfs.append(field_match_objective(func[1], func[0], weight=1))
        for comps, fprime, fun in self.udfs:
            if not callable(fprime):
                raise ValueError("The derivative function is not callable")
            if not callable(fun):
                raise ValueError("The objective function is not callable")
            for c in comps:
                self.add_component(c)

    def add_component(self, component="Ex"):
        if component in self.forward_dfts:
            return
        self.forward_dfts[component] = self.forward_simulation.add_dft_fields(
            center=self.center, size=self.size, frequency=[self.frequency], field_component=component)
        # the reference names the datasets "<component> adjoint"
        # (ffip/simulation.py:711-721), so two Adjoint_Source objects of one
        # adjoint simulation would write the same datasets and every one of
        # them would run with the last one's amplitudes; a later source here
        # gets a numbered suffix instead (the first keeps the reference's name)
        suffix = component + " adjoint"
        used = {getattr(src, "amplitude_dataset_name", None) for src in getattr(self.adjoint_simulation, "sources", ())}
        n = 1
        while "inhom source amplitude %s" % suffix in used:
            suffix = "%s adjoint %d" % (component, n)
            n += 1
        self.adjoint_sources[component] = Inhom_Source(function=self.function, frequency=self.frequency, amplitude=None,
                                                       center=self.center, size=self.size, dim=self.dim,
                                                       field_component=component, suffix=suffix)
        self.adjoint_simulation.add_source(self.adjoint_sources[component])

    @property
    def shape(self):
        return (int(self.dim.z), int(self.dim.y), int(self.dim.x))

    @property
    def numel(self):
        return int(self.dim.prod())

    def eval_functionals_and_set_sources(self):
        for c in self.forward_dfts:
            self.adjoint_sources[c].amplitude = np.zeros(self.shape, dtype=complex)
            self.forward_fields[c] = self.forward_dfts[c](self.frequency, self.z, self.y, self.x).reshape(self.shape)
        res = 0
        for comps, fprime, fun in self.udfs:
            args = [self.forward_fields[c] for c in comps]
            res = res + fun(*args)
            ders = fprime(*args)
            for i, c in enumerate(comps):
                self.adjoint_sources[c].amplitude += ders[i]
        return res


class Adjoint_Flux:
    """Adjoint sources of a flux objective (simulation.py:585-645)."""

    def __init__(self, adjoint_simulation, forward_simulation, function, fluxes=(), frequency=1.0, scale=1):
        self.adjoint_simulation, self.forward_simulation = adjoint_simulation, forward_simulation
        self.frequency, self.scale = float(frequency), float(scale)
        self.fluxes = list(fluxes)
        self.e_adjoint_sources, self.m_adjoint_sources = [], []
        for i, flux in enumerate(self.fluxes):
            if flux.frequency.size > 1:
                raise ValueError("Fluxes used in Adjoint_Flux cannot have more than 1 frequency")
            for comp, lst in ((flux.e1_str, self.e_adjoint_sources), (flux.h2_str, self.m_adjoint_sources)):
                lst.append(Inhom_Source(function=function, frequency=frequency, amplitude=None, center=flux.center,
                                        size=flux.size, dim=flux.get_len(scale=scale), field_component=comp,
                                        suffix="flux %d %s adjoint" % (i, comp)))
            adjoint_simulation.add_source(self.e_adjoint_sources[-1])
            adjoint_simulation.add_source(self.m_adjoint_sources[-1])

    def eval_functionals_and_set_sources(self):
        res = 0
        for i, flux in enumerate(self.fluxes):
            res += flux.get_values(scale=self.scale)
            e1, h2 = flux.get_fields(scale=self.scale)
            w = flux.get_int_weights(scale=self.scale)
            self.e_adjoint_sources[i].amplitude = np.conj(h2[0, ...]) * w
            self.m_adjoint_sources[i].amplitude = -np.conj(e1[0, ...]) * w
        return res


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def frequency_factor(frequency, dt=None):
    """The factor that turns E_fwd E_adj / norm into d F / d epsilon.  The
    reference uses the continuous 2 pi j f (ffip/simulation.py:858); the
    leap-frog E update, (E^{n+1} - E^n)/dt with the pulse sampled at half
    steps, makes it 2 j sin(pi f dt) / dt exactly (dt given)."""
    if dt is None:
        return 2j * pi * frequency
    return 2j * np.sin(pi * frequency * dt) / dt


def sensitivity_scatter(factor, norm, fwd, adj, deps, x, y, z, gx, gy, gz):
    """Re(factor fwd adj deps / norm) at points (x, y, z), scattered onto the
    grid gx x gy x gz with the transpose of trilinear interpolation; on the GPU
    (ffip_sensitivity)."""
    lib = native.load()
    n = int(np.size(x))
    c2 = lambda a: np.ascontiguousarray(np.stack([np.real(a), np.imag(a)], axis=-1).reshape(-1), dtype=np.float64)
    f, a, d = c2(np.broadcast_to(fwd, (n,))), c2(np.broadcast_to(adj, (n,))), c2(np.broadcast_to(deps, (n,)))
    xyz = np.ascontiguousarray(np.stack([np.ravel(x), np.ravel(y), np.ravel(z)], axis=-1), dtype=np.float64)
    gx, gy, gz = (np.ascontiguousarray(np.asarray(v, dtype=np.float64)) for v in (gx, gy, gz))
    out = np.zeros((gz.size, gy.size, gx.size))
    norm, factor = complex(norm), complex(factor)
    rc = lib.ffip_sensitivity(factor.real, factor.imag, norm.real, norm.imag, _dptr(f), _dptr(a), _dptr(d), _dptr(xyz), n,
                              _dptr(gx), gx.size, _dptr(gy), gy.size, _dptr(gz), gz.size, _dptr(out))
    if rc != 0:
        raise native.FfipError(lib.ffip_last_error().decode())
    return out


def _dft_at_points(dft, f, x, y, z):
    """A DFT monitor's values at frequency f and points (x, y, z): where every
    point is a node of the monitor's output grid (the design box's own grid
    points are), read directly -- the linear interpolant returns the node's
    value there -- else through the interpolant."""
    def index(grid, q):
        grid = np.asarray(grid, dtype=float)
        i = np.clip(np.searchsorted(grid, q), 0, grid.size - 1)
        j = np.clip(i - 1, 0, grid.size - 1)
        i = np.where(np.abs(grid[j] - q) < np.abs(grid[i] - q), j, i)
        return i, np.all(np.abs(grid[i] - q) <= 1e-9 * max(1.0, float(np.abs(grid).max())))
    rf, rz, ry, rx, rv = dft.raw
    fi = np.flatnonzero(np.asarray(rf) == f)
    ix, okx = index(rx, x)
    iy, oky = index(ry, y)
    iz, okz = index(rz, z)
    if fi.size and okx and oky and okz:
        return rv[fi[0], iz, iy, ix]
    pts = np.stack((f * np.ones(np.shape(z)), z, y, x), axis=-1)
    return dft.get_interpolant(method="linear", bounds_error=True)(pts)


class Adjoint_Volume:
    """Design region and its sensitivity (simulation.py:759-915)."""

    def __init__(self, adjoint_simulation, forward_simulation, frequency=1.0, center=None, size=None, dim=None, density=None,
                 medium1=None, medium2=None, epsilon_fun=None, epsilon_der=None, e_sus=(), norm=1, geometry=None):
        """norm: the spectrum sum_n g(t_n) exp(-2 pi j f t_n) of the pulse g of
        the adjoint sources at this frequency (the adjoint field carries that
        pulse; when the forward pulse differs, the forward one is not the
        right divisor).

        geometry (rebuild-only): the design box of another Adjoint_Volume
        of the same forward simulation (another frequency); it is then added
        to the adjoint simulation only, so that the forward simulation holds
        the design box once."""
        self.adjoint_simulation, self.forward_simulation = adjoint_simulation, forward_simulation
        self.frequency = float(frequency)
        self.center = (center if center is not None else Vector3()).copy()
        self.size = (size if size is not None else Vector3()).copy()
        dim = dim if dim is not None else Vector3()
        self.dim = dim.round()
        self.norm = complex(norm)
        medium1 = medium1 if medium1 is not None else Medium()
        medium2 = medium2 if medium2 is not None else Medium()
        if epsilon_fun is None:
            e1, e2 = medium1.get_epsilon(self.frequency), medium2.get_epsilon(self.frequency)
            self.epsilon_fun = lambda rho: e1 * rho + (1 - rho) * e2
            self.epsilon_der = lambda rho: e1 - e2
            self.medium1, self.medium2 = deepcopy(medium1), deepcopy(medium2)
            if geometry is None:
                geometry = Two_Medium_Box(size=self.size, center=self.center, dim=dim, density=density, medium1=medium1,
                                          medium2=medium2, suffix="adjoint")
        else:
            self.epsilon_der, self.epsilon_fun = epsilon_der, epsilon_fun
            if geometry is None:
                geometry = General_Medium_Box(size=self.size, center=self.center, dim=dim, frequency=frequency,
                                              density=density, epsilon_fun=epsilon_fun, e_sus=e_sus, suffix="adjoint")
        shared = geometry is not None and any(g is geometry for g in forward_simulation.geometry)
        self.geom = geometry
        # a shared adjoint simulation (one broadband adjoint run for several
        # frequencies' volumes) holds the design box once, too
        if not any(g is geometry for g in adjoint_simulation.geometry):
            adjoint_simulation.add_geometry(self.geom)
        if not shared:
            forward_simulation.add_geometry(self.geom)
        comps = ["Ex", "Ey", "Ez"]
        self.forward_dfts = [forward_simulation.add_dft_fields(center=self.center, size=self.size, frequency=[frequency],
                                                               field_component=c) for c in comps]
        self.adjoint_dfts = [adjoint_simulation.add_dft_fields(center=self.center, size=self.size, frequency=[frequency],
                                                               field_component=c) for c in comps]
        self.geom_infos = [forward_simulation.request_geom_info(geom=self.geom, field_component=c) for c in comps]

    def forward_dft(self, field_component="Ex"):
        return self.forward_dfts["xyz".index(field_component[1])]

    def adjoint_dft(self, field_component="Ex"):
        return self.adjoint_dfts["xyz".index(field_component[1])]

    def design_points(self, component):
        """Exact physical coordinates of the grid points of E component
        `component` (0..2) strictly inside the design box (the reference's
        geometry-info coordinates are truncated to integers)."""
        dx2 = self.forward_simulation.dx / 2
        p1 = (self.center - self.size / 2) / dx2
        p2 = (self.center + self.size / 2) / dx2
        axes = []
        for a in range(3):
            par = 1 if a == component else 0
            lo = int(np.floor(p1[a])) + 1
            hi = int(np.ceil(p2[a])) - 1
            c = np.arange(lo, hi + 1)
            c = c[(c & 1) == par]
            c = c[(c > p1[a]) & (c < p2[a])]
            axes.append(c * dx2)
        Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
        return X.ravel(), Y.ravel(), Z.ravel()

    def get_sensitivity(self, exact=False):
        """dF/drho on the density grid: Re(2 pi j f E_fwd E_adj deps/drho / norm)
        at every E point of the design box, transposed through the trilinear
        density interpolation (simulation.py:841-869), on the GPU.  exact=True
        uses the leap-frog factor 2 j sin(pi f dt)/dt instead of 2 pi j f."""
        rho_interp = RegularGridInterpolator((self.z, self.y, self.x), self.density, bounds_error=True)
        dt = self.forward_simulation.dx * self.forward_simulation.courant
        factor = frequency_factor(self.frequency, dt if exact else None)
        res = 0
        for i in range(3):
            x, y, z = self.design_points(i)
            fwd = _dft_at_points(self.forward_dfts[i], self.frequency, x, y, z)
            adj = _dft_at_points(self.adjoint_dfts[i], self.frequency, x, y, z)
            deps = self.epsilon_der(rho_interp(np.stack((z, y, x), axis=-1)))
            res = res + sensitivity_scatter(factor, self.norm, fwd, adj, np.asarray(deps, dtype=complex), x, y, z,
                                            self.x, self.y, self.z)
        return np.reshape(res, self.shape)

    def get_sensitivity2(self):
        """The same correlation evaluated at the density nodes (simulation.py:871-883)."""
        pts = np.stack(np.meshgrid(self.frequency, self.z, self.y, self.x, indexing="ij"), axis=-1)
        res = 0
        for i in range(3):
            fwd = self.forward_dfts[i].get_interpolant(method="linear", bounds_error=True)(pts)
            adj = self.adjoint_dfts[i].get_interpolant(method="linear", bounds_error=True)(pts)
            res = res + 2j * pi * self.frequency * fwd * adj / self.norm
        return np.real(np.reshape(res, self.shape) * self.epsilon_der(self.density))

    @property
    def x(self):
        return self.geom.x

    @property
    def y(self):
        return self.geom.y

    @property
    def z(self):
        return self.geom.z

    @property
    def p1(self):
        return self.center - self.size / 2

    @property
    def density(self):
        return self.geom.density

    @density.setter
    def density(self, val):
        self.geom.density = val

    @property
    def numel(self):
        return int(self.dim.prod())

    @property
    def shape(self):
        return self.geom.shape
