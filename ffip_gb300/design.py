"""Design-loop layer: one objective evaluation = forward run + adjoint run(s)
on the GPU stepper, exposed to PyTorch as a differentiable function of the
design density.

The reference's optimisation scripts repeat, per design iteration
(scripts/optimizations/*, ffip/simulation.py:648-915):

    forward.run(stop); F = adjoint_source.eval_functionals_and_set_sources()
    adjoint.run(stop); grad = adjoint_volume.get_sensitivity()

`AdjointProblem` runs the same sequence with the device simulations kept
between iterations (Simulation.run(keep=True): the density and the adjoint
source datasets are updated in place), and `DensityObjective` wraps it as a
torch.autograd.Function: forward returns F(rho), backward runs the adjoint
simulations and returns dF/drho.  Only DFT fields are stored: the objectives
are frequency-domain, so no time history is checkpointed.

Several (adjoint simulation, adjoint sources, adjoint volume) terms may share
one forward simulation, as the reference's multi-frequency scripts do (one
adjoint run per frequency); F and the gradient are summed over the terms.
`BroadbandAdjoint` is the rebuild's alternative for an objective over several
frequencies: one adjoint run whose source spectrum equals every frequency's
adjoint amplitude at once.
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

from .simulation import Adjoint_Source
from .source import Gaussian1, Inhom_Source


class AdjointTerm:
    """One adjoint simulation with its sources (Adjoint_Source / Adjoint_Flux
    objects) and the Adjoint_Volume that correlates it with the forward run."""

    def __init__(self, adjoint_simulation, sources: Sequence, volume):
        self.adjoint_simulation = adjoint_simulation
        self.sources = list(sources)
        self.volume = volume

    def evaluate(self) -> complex:
        """Objective share of this term; sets its adjoint sources."""
        F = 0.0
        for s in self.sources:
            F = F + s.eval_functionals_and_set_sources()
        return F

    def sensitivity(self, exact: bool) -> np.ndarray:
        return self.volume.get_sensitivity(exact=exact)


class _SourceCollector:
    """Stands in for the adjoint simulation while per-frequency
    Adjoint_Source objects are built for a BroadbandAdjoint: it keeps their
    inhomogeneous sources, which never run themselves."""

    def __init__(self):
        self.sources = []

    def add_source(self, src):
        self.sources.append(src)


class SignedInhomSource(Inhom_Source):
    """An inhomogeneous source whose amplitude dataset holds signed real
    values and whose phase dataset is zero, so that each dipole's amplitude
    carries the sign (Simulation::set_inhom_source multiplies the dataset
    value into the dipole amplitude, src/simulation.cpp:284-336; the
    reference's own Inhom_Source writes |a| and arg(a), ffip/source.py:126-129,
    which turns a sign into a time shift of the pulse)."""

    def dump(self, datasets):
        datasets[self.amplitude_dataset_name] = np.ascontiguousarray(np.real(self.amplitude).ravel(), dtype=np.float64)
        datasets[self.phase_dataset_name] = np.zeros(self.amplitude.size)


class BroadbandAdjoint:
    """One adjoint run for an objective over m frequencies f_i.

    The reference runs one adjoint simulation per frequency: at each
    adjoint-source point p it places a pulse g whose amplitude |a_pi| and
    time shift (from arg a_pi) make its spectrum a_pi G(f_i) at f_i, where
    a_pi = dF/dE*(p, f_i) and G is the pulse's spectrum
    (ffip/simulation.py:728-753, src/simulation.cpp:284-336).  Here every
    point gets K = 2m copies of the pulse delayed by tau_k = k T (multiples of
    dt, so that each copy's sampled spectrum is exactly e^{-2 pi j f tau_k} G(f))
    with signed real amplitudes b_pk solving

        sum_k b_pk e^{-2 pi j f_i tau_k} = a_pi      for every i,

        (2m real equations in 2m unknowns; T is chosen to make the matrix
        well conditioned), so that the one run's source spectrum at every f_i is
    a_pi G(f_i): the adjoint DFT fields at each f_i are those of the
    per-frequency run, and each frequency's Adjoint_Volume divides by G(f_i)
    (norm(f)).  One adjoint run replaces m.

    Usage: build the per-frequency Adjoint_Source objects with source() and
    the Adjoint_Volume objects on `adjoint_simulation` with norm=norm(f), add
    the volumes with add_volume(), and pass the object as a term of an
    AdjointProblem."""

    def __init__(self, adjoint_simulation, forward_simulation, function: Gaussian1, frequencies, dt: float):
        self.adjoint_simulation = adjoint_simulation
        self.forward_simulation = forward_simulation
        self.function = function
        self.frequencies = [float(f) for f in frequencies]
        self.dt = float(dt)
        self.sources: List[Adjoint_Source] = []
        self.volumes = []
        self._collector = _SourceCollector()
        self._signed = {}  # (component, center, size, dim) -> K SignedInhomSource on the adjoint simulation
        m = len(self.frequencies)
        if m < 1 or len(set(self.frequencies)) != m:
            raise ValueError("BroadbandAdjoint needs distinct frequencies")
        self.shifts, self._M = self._design(np.asarray(self.frequencies), self.dt)

    @staticmethod
    def _matrix(f, tau):
        E = np.exp(-2j * np.pi * f[:, None] * tau[None, :])
        return np.concatenate([E.real, E.imag])

    @classmethod
    def _design(cls, f, dt):
        """Delays k T (T a multiple of dt, K = 2m of them) that make the
        matrix of the equations best conditioned."""
        K = 2 * f.size
        span = 2.0 / max(np.min(np.diff(np.sort(f))) if f.size > 1 else f[0], 1e-12)
        best = None
        for T in np.arange(dt, span + dt, dt):
            c = np.linalg.cond(cls._matrix(f, np.arange(K) * T))
            if best is None or c < best[0] - 1e-9:
                best = (c, T)
        if best is None or not np.isfinite(best[0]) or best[0] > 1e6:
            raise ValueError("no delay spacing separates these frequencies")
        tau = np.arange(K) * best[1]
        return tau, cls._matrix(f, tau)

    def source(self, frequency, **kwargs) -> Adjoint_Source:
        """An Adjoint_Source at one of the frequencies (the arguments of
        Adjoint_Source after the function); its amplitudes feed the
        broadband sources."""
        frequency = float(frequency)
        if frequency not in self.frequencies:
            raise ValueError("frequency %g is not one of the broadband adjoint's frequencies" % frequency)
        s = Adjoint_Source(self._collector, self.forward_simulation, self.function, frequency=frequency, **kwargs)
        self.sources.append(s)
        for comp, inh in s.adjoint_sources.items():
            key = self._key(comp, inh)
            if key in self._signed:
                continue
            srcs = []
            for k, tau in enumerate(self.shifts):
                fn = Gaussian1(self.function.frequency, cutoff=self.function.cutoff, start_time=self.function.start_time + tau)
                src = SignedInhomSource(function=fn, amplitude=None, frequency=self.function.frequency, center=inh.center,
                                        size=inh.size, dim=inh.dim, field_component=comp,
                                        suffix="%s broadband %d %d" % (comp, len(self._signed), k))
                self.adjoint_simulation.add_source(src)
                srcs.append(src)
            self._signed[key] = srcs
        return s

    @staticmethod
    def _key(comp, inh):
        return (comp, tuple(inh.center.get_json()), tuple(inh.size.get_json()), tuple(inh.dim.get_json()))

    def norm(self, frequency) -> complex:
        """G(f): the sampled spectrum of the undelayed pulse, sum over the
        pulse's time samples of g(t) e^{-2 pi j f t} -- the divisor of the
        Adjoint_Volume at f."""
        g = self.function
        t = np.arange(g.start_time, g.end_time, self.dt)
        return complex(np.sum(np.exp(-2j * np.pi * float(frequency) * t) * g(t)))

    def add_volume(self, volume):
        self.volumes.append(volume)

    def evaluate(self) -> complex:
        """Objective share (every per-frequency source's functionals) and the
        broadband sources' amplitudes from their adjoint amplitudes."""
        F = 0.0
        for s in self.sources:
            F = F + s.eval_functionals_and_set_sources()
        m = len(self.frequencies)
        for key, srcs in self._signed.items():
            shape = srcs[0].shape
            A = np.zeros((m,) + shape, dtype=complex)
            for s in self.sources:
                i = self.frequencies.index(s.frequency)
                for comp, inh in s.adjoint_sources.items():
                    if self._key(comp, inh) == key:
                        A[i] += inh.amplitude
            rhs = np.concatenate([A.real.reshape(m, -1), A.imag.reshape(m, -1)])
            b = np.linalg.solve(self._M, rhs)
            for k, src in enumerate(srcs):
                src.amplitude = b[k].reshape(shape)
        return F

    def sensitivity(self, exact: bool) -> np.ndarray:
        g = 0
        for v in self.volumes:
            g = g + v.get_sensitivity(exact=exact)
        return g


class AdjointProblem:
    """Objective and density gradient of one design region.

    forward_simulation: Simulation that holds the design geometry (every
    term's Adjoint_Volume adds it) and the forward DFT monitors.
    terms: AdjointTerm list.  stop: stop condition of every run.
    exact: use the leap-frog factor 2j sin(pi f dt)/dt in the gradient
    (True) or the reference's 2 pi j f (False)."""

    def __init__(self, forward_simulation, terms: List[AdjointTerm], stop, exact: bool = True):
        if not terms:
            raise ValueError("an adjoint problem needs at least one term")
        self.forward_simulation = forward_simulation
        self.terms = list(terms)
        self.stop = stop
        self.exact = exact
        self.value = None
        self._pending = False

    @property
    def density(self) -> np.ndarray:
        t = self.terms[0]
        return (t.volumes[0] if isinstance(t, BroadbandAdjoint) else t.volume).density

    def forward(self, rho: np.ndarray) -> float:
        """Sets the density of every term's design box, runs the forward
        simulation and evaluates the objective (the adjoint sources are set)."""
        rho = np.asarray(rho, dtype=np.float64)
        for t in self.terms:
            for v in (t.volumes if isinstance(t, BroadbandAdjoint) else [t.volume]):
                v.density = rho
        self.forward_simulation.run(self.stop, keep=True)
        F = 0.0
        for t in self.terms:
            F = F + t.evaluate()
        # (a flux objective is an array over its frequencies: their sum)
        self.value = float(np.real(np.sum(F)))
        self._pending = True
        return self.value

    def gradient(self) -> np.ndarray:
        """dF/drho at the density of the last forward(): one adjoint run per term."""
        if not self._pending:
            raise RuntimeError("gradient() needs a forward() first")
        g = 0
        for t in self.terms:
            t.adjoint_simulation.run(self.stop, keep=True)
            g = g + t.sensitivity(self.exact)
        return np.asarray(g, dtype=np.float64)

    def value_and_gradient(self, rho: np.ndarray):
        F = self.forward(rho)
        return F, self.gradient()

    def release(self):
        self.forward_simulation.release()
        for t in self.terms:
            t.adjoint_simulation.release()


def _torch():
    import torch
    return torch


class DensityObjective:
    """torch.autograd.Function F(rho) of an AdjointProblem:

        F = DensityObjective.apply(rho, problem)
        F.backward()          # rho.grad = dF/drho from the adjoint run(s)

    rho is any float tensor with the design box's shape (z, y, x); the
    simulations run in fp64 or fp32 as their Simulation objects ask."""

    _fn = None

    @classmethod
    def apply(cls, rho, problem: AdjointProblem):
        if cls._fn is None:
            torch = _torch()

            class _Fn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, r, prob):
                    rho = r.detach().cpu().double().numpy().copy()
                    F = prob.forward(rho)
                    ctx.problem = prob
                    ctx.rho = rho
                    ctx.meta = (r.dtype, r.device)
                    return torch.tensor(F, dtype=r.dtype, device=r.device)

                @staticmethod
                def backward(ctx, gF):
                    dtype, device = ctx.meta
                    prob = ctx.problem
                    # another forward() since this one (a line search): redo this one
                    if not np.array_equal(np.asarray(prob.density, dtype=np.float64), ctx.rho):
                        prob.forward(ctx.rho)
                    g = torch.from_numpy(prob.gradient()).to(device=device, dtype=dtype)
                    return gF * g, None

            cls._fn = _Fn
        return cls._fn.apply(rho, problem)
