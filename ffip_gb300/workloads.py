"""Seeded synthetic workloads in the reference's config schema.

``dispersive_spheres(n=256)`` is the dispersive-scattering workload the
throughput figures are quoted on: an n^3-cell box, dx = 1, Courant 0.5,
CPML of n/16 cells (order 3, sigma_max = -(m+1) ln(1e-8) / (2 d)), background
vacuum, 64 spheres (centres uniform in the non-CPML interior, radii uniform
4-16 cells scaled by n/256) of which half use one 2-pole Lorentz medium
(eps_inf 2, delta-eps U(0.5, 3), omega_0 U(0.05, 0.2), gamma U(0.001, 0.02))
and half one Drude medium (omega_p U(0.3, 1.0), gamma U(0.005, 0.05)); an Ex
current sheet at z index 3n/32 with a Gaussian1 pulse at f = 0.1; a DFT volume
monitor of Ex, n/2 x n/2 x n/8 cells, centred, at 5 frequencies in
[0.06, 0.14]; 4000 steps at n = 256 (scaled by n/256 below that).

Angular rates: omega_0, omega_p and gamma are taken as angular (rad per unit
time), so the reference's "frequency"/"gamma" parameters (which it multiplies
by 2 pi, src/medium.cpp:98-108) are omega / (2 pi).  Read as plain frequency
parameters, Drude plasma frequencies above about 0.45 make the reference's
own ADE update diverge at Courant 0.5.
"""
from __future__ import annotations

import math

import numpy as np

TWO_PI = 2 * math.pi


def medium(eps=1.0, mu=1.0, esus=()):
    return {"epsilon": eps, "mu": mu, "electric conductivity": 0.0, "magnetic conductivity": 0.0,
            "electric susceptibility": list(esus), "magnetic susceptibility": []}


def sigma_max(order: int, thickness: float, R: float = 1e-8) -> float:
    """sigma_max for a polynomial CPML of given order and reflection R."""
    return -(order + 1) * math.log(R) / (2 * thickness)


def dispersive_spheres(n: int = 256, steps: int | None = None, seed: int = 2024, precision: str = "fp32",
                       engine: str = "auto") -> dict:
    rng = np.random.default_rng(seed)
    scale = n / 256.0
    pml = max(2, int(round(16 * scale)))
    half = n / 2.0
    lor = medium(2.0, esus=[{"type": "Lorentz", "frequency": rng.uniform(0.05, 0.2) / TWO_PI,
                             "gamma": rng.uniform(0.001, 0.02) / TWO_PI, "amplitude": rng.uniform(0.5, 3.0)}
                            for _ in range(2)])
    dru = medium(1.0, esus=[{"type": "Drude", "frequency": rng.uniform(0.3, 1.0) / TWO_PI,
                             "gamma": rng.uniform(0.005, 0.05) / TWO_PI, "amplitude": 1.0}])
    geoms = []
    lo, hi = -half + pml, half - pml
    for s in range(64):
        r = rng.uniform(4, 16) * scale
        c = rng.uniform(lo, hi, size=3)
        geoms.append({"type": "sphere", "center": [float(v) for v in c], "radius": float(r),
                      "medium": lor if s % 2 == 0 else dru})
    z_sheet = -half + 24 * scale
    cfg = {
        "courant number": 0.5, "resolution": 1.0, "size": [float(n)] * 3,
        "input file": "input.h5", "fields output file": "output.h5",
        "default material": medium(), "progress interval": 1e9,
        "PML": [{"thickness": float(pml), "k max": 1.0, "sigma max": sigma_max(3, pml), "order": 3}],
        "geometry": geoms,
        "sources": [{"type": "volume source", "center": [0.0, 0.0, z_sheet], "size": [n - 2.0 * pml, n - 2.0 * pml, 0.0],
                     "amplitude": 1.0, "field component": "Ex",
                     "function": {"type": "Gaussian1", "frequency": 0.1, "cutoff": 4.0, "start time": 0.0}}],
        "fields output": [{"type": "volume fields dft", "center": [0.0, 0.0, 0.0], "size": [n / 2.0, n / 2.0, n / 8.0],
                           "frequency": [float(f) for f in np.linspace(0.06, 0.14, 5)], "field component": "Ex",
                           "output group": "volume fields dft 0"}],
        "precision": precision, "engine": engine,
    }
    nsteps = steps if steps is not None else max(100, int(round(4000 * scale)))
    cfg["stop condition"] = {"type": "time", "time": nsteps * 0.5}
    return cfg


def vacuum_point(n: int = 64, steps: int = 1000, seed: int = 7, precision: str = "fp64", engine: str = "auto") -> dict:
    """n^3 vacuum box, 8-cell CPML (order 3, R = 1e-8), one Ez point current at
    a seeded interior cell (Gaussian1, f = 0.1), DFT Ez plane at z = +n/4 at
    3 frequencies."""
    rng = np.random.default_rng(seed)
    pml = 8
    half = n / 2
    c = rng.integers(int(-half + pml + 2), int(half - pml - 2), size=3)
    return {
        "courant number": 0.5, "resolution": 1.0, "size": [float(n)] * 3,
        "input file": "input.h5", "fields output file": "output.h5", "default material": medium(),
        "PML": [{"thickness": float(pml), "k max": 1.0, "sigma max": sigma_max(3, pml), "order": 3}],
        "sources": [{"type": "volume source", "center": [float(c[0]), float(c[1]), float(c[2]) + 0.5], "size": [0.0, 0.0, 0.0],
                     "amplitude": 1.0, "field component": "Ez",
                     "function": {"type": "Gaussian1", "frequency": 0.1, "cutoff": 4.0, "start time": 0.0}}],
        "fields output": [{"type": "volume fields dft", "center": [0.0, 0.0, n / 4.0], "size": [float(n), float(n), 0.0],
                           "frequency": [0.08, 0.1, 0.12], "field component": "Ez", "output group": "volume fields dft 0"}],
        "stop condition": {"type": "time", "time": steps * 0.5},
        "precision": precision, "engine": engine,
    }


def large_design(n: int = 512, nz: int = 384, pml: int = 24, design=(256, 32), nfreq: int = 16, steps: int = 20000,
                 seed: int = 2024, precision: str = "fp32", engine: str = "auto"):
    """The large design workload (one forward simulation of the
    surrogate-screened design loop at scale): an n x n x nz cell box (dx = 1,
    Courant 0.5) with a `pml`-cell CPML; a Drude metal backplane (omega_p
    0.8, gamma 0.02, angular rates as in dispersive_spheres) 8 cells thick
    across the interior, 8 cells above the lower CPML; on it a design box of
    design[0] x design[0] x design[1] cells whose density (nodes at every
    cell corner) is seeded filtered noise (sigma = 4 nodes) between a 2-pole
    Lorentz design material (the dispersive_spheres recipe) and vacuum; an Ex
    current sheet (Gaussian1, f = 0.1) half-way up; three 256 x 256 DFT
    planes (Ex and Ey at one height, Ex at another) at `nfreq` frequencies in
    [0.06, 0.14]; `steps` time steps.  Returns (config, datasets)."""
    rng = np.random.default_rng(seed)
    dn, dz = design
    lor = medium(2.0, esus=[{"type": "Lorentz", "frequency": rng.uniform(0.05, 0.2) / TWO_PI,
                             "gamma": rng.uniform(0.001, 0.02) / TWO_PI, "amplitude": rng.uniform(0.5, 3.0)}
                            for _ in range(2)])
    dru = medium(1.0, esus=[{"type": "Drude", "frequency": 0.8 / TWO_PI, "gamma": 0.02 / TWO_PI, "amplitude": 1.0}])
    z_lo = -nz / 2.0 + pml
    inner = n - 2.0 * pml
    z_plate = z_lo + 8 + 4.0
    z_design = z_lo + 16 + dz / 2.0
    rho = filtered_noise((dz + 1, dn + 1, dn + 1), 4.0, seed)
    freqs = [float(f) for f in np.linspace(0.06, 0.14, nfreq)]
    cfg = {
        "courant number": 0.5, "resolution": 1.0, "size": [float(n), float(n), float(nz)],
        "input file": "input.h5", "fields output file": "output.h5",
        "default material": medium(), "progress interval": 1e9,
        "PML": [{"thickness": float(pml), "k max": 1.0, "sigma max": sigma_max(3, pml), "order": 3}],
        "geometry": [{"type": "box", "center": [0.0, 0.0, z_plate], "size": [inner, inner, 8.0], "medium": dru},
                     {"type": "two medium box", "center": [0.0, 0.0, z_design], "size": [float(dn), float(dn), float(dz)],
                      "dimension": [dn + 1, dn + 1, dz + 1], "density dataset": "two medium box 0",
                      "medium1": lor, "medium2": medium()}],
        "sources": [{"type": "volume source", "center": [0.0, 0.0, 0.0], "size": [inner, inner, 0.0],
                     "amplitude": 1.0, "field component": "Ex",
                     "function": {"type": "Gaussian1", "frequency": 0.1, "cutoff": 4.0, "start time": 0.0}}],
        "fields output": [{"type": "volume fields dft", "center": [0.0, 0.0, zc], "size": [256.0, 256.0, 0.0],
                           "frequency": freqs, "field component": comp, "output group": "volume fields dft %d" % i}
                          for i, (comp, zc) in enumerate((("Ex", nz / 4.0), ("Ey", nz / 4.0), ("Ex", nz / 2.0 - pml - 16.0)))],
        "stop condition": {"type": "time", "time": steps * 0.5},
        "precision": precision, "engine": engine,
    }
    return cfg, {"two medium box 0": rho.ravel()}


def filtered_noise(shape, sigma, seed):
    """Seeded uniform noise, Gaussian-filtered (sigma in nodes), min-max
    rescaled to [0, 1]: the design-density recipe of the adjoint workload."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    r = gaussian_filter(rng.uniform(0, 1, size=shape), sigma=sigma, mode="reflect")
    return (r - r.min()) / (r.max() - r.min())


def adjoint_design(size=(192, 160), design=(96, 24), pml=16, freqs=(0.09, 0.1, 0.11), steps=5000, nprobe=4,
                   seed=2024, precision="fp32", exact=True, broadband=True, eps_design=12.0):
    """The adjoint-gradient workload: a size[0] x size[0] x size[1] cell box
    (dx = 1, Courant 0.5) with a `pml`-cell CPML; a design box of
    design[0] x design[0] x design[1] cells centred at the origin whose
    density (nodes at every cell corner: (design + 1) per axis) is seeded
    filtered noise (sigma = 3 nodes), eps = 1 + 11 rho (medium1 eps 12,
    medium2 vacuum; eps_design replaces the 12); an Ex current sheet (Gaussian1, f = 0.1) half-way
    between the lower CPML and the design box; objective F = sum over
    `nprobe` seeded probe cells above the design box and over `freqs` of
    |Ex|^2.  One forward run and, with broadband=True, one adjoint run for
    all frequencies (design.BroadbandAdjoint), else one adjoint run per
    frequency as the reference's scripts do; `steps` time steps each.
    Returns (AdjointProblem, rho0)."""
    from . import design as D
    from .geom import Medium, Vector3
    from .simulation import Adjoint_Source, Adjoint_Volume, Simulation, field_match_objective, run_until_time
    from .source import Gaussian1, Source
    from .simulation import PML
    n, nz = size
    dn, dz = design
    rng = np.random.default_rng(seed)
    V = Vector3
    pmls = [PML(thickness=pml, sigma_max=sigma_max(3, pml))]
    z_lo = -nz / 2 + pml
    z_sheet = float(np.round((z_lo + (-dz / 2)) / 2))
    fwd_func = Gaussian1(0.1, cutoff=4, start_time=0.0)
    fwd = Simulation(size=V(n, n, nz), resolution=1, pmls=pmls, precision=precision,
                     sources=[Source(function=fwd_func, center=V(0, 0, z_sheet), size=V(n - 2 * pml, n - 2 * pml, 0),
                                     field_component="Ex")])
    probes = [(float(rng.integers(-dn // 3, dn // 3)) + 0.5, float(rng.integers(-dn // 3, dn // 3)),
               float(rng.integers(dz // 2 + 8, nz / 2 - pml - 8))) for _ in range(nprobe)]
    rho0 = filtered_noise((dz + 1, dn + 1, dn + 1), 3.0, seed)
    dt = 0.5
    if broadband:
        adj = Simulation(size=V(n, n, nz), resolution=1, pmls=pmls, precision=precision)
        bb = D.BroadbandAdjoint(adj, fwd, Gaussian1(0.1, cutoff=4, start_time=0.0), freqs, dt)
        geom = None
        for f in freqs:
            for p in probes:
                bb.source(f, center=V(*p), size=V(0, 0, 0), dim=V(1, 1, 1),
                          udfs=[field_match_objective(np.zeros((1, 1, 1)), "Ex", weight=1.0)])
            vol = Adjoint_Volume(adj, fwd, frequency=f, center=V(0, 0, 0), size=V(dn, dn, dz), dim=V(dn + 1, dn + 1, dz + 1),
                                 density=rho0, medium1=Medium(epsilon=eps_design), medium2=Medium(), norm=bb.norm(f), geometry=geom)
            geom = vol.geom
            bb.add_volume(vol)
        return D.AdjointProblem(fwd, [bb], run_until_time(steps * dt), exact=exact), rho0
    terms, geom = [], None
    for f in freqs:
        adj = Simulation(size=V(n, n, nz), resolution=1, pmls=pmls, precision=precision)
        adj_func = Gaussian1(0.1, cutoff=4, start_time=0.5 / f)
        srcs = [Adjoint_Source(adj, fwd, function=adj_func, frequency=f, center=V(*p), size=V(0, 0, 0), dim=V(1, 1, 1),
                               udfs=[field_match_objective(np.zeros((1, 1, 1)), "Ex", weight=1.0)]) for p in probes]
        # the adjoint field carries the adjoint pulse: normalise by its spectrum
        t = np.arange(adj_func.start_time, adj_func.end_time, dt)
        norm = np.sum(np.exp(-2j * np.pi * f * t) * adj_func(t))
        vol = Adjoint_Volume(adj, fwd, frequency=f, center=V(0, 0, 0), size=V(dn, dn, dz), dim=V(dn + 1, dn + 1, dz + 1),
                             density=rho0, medium1=Medium(epsilon=eps_design), medium2=Medium(), norm=norm, geometry=geom)
        geom = vol.geom
        terms.append(D.AdjointTerm(adj, srcs, vol))
    return D.AdjointProblem(fwd, terms, run_until_time(steps * dt), exact=exact), rho0
