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
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np


class AdjointTerm:
    """One adjoint simulation with its sources (Adjoint_Source / Adjoint_Flux
    objects) and the Adjoint_Volume that correlates it with the forward run."""

    def __init__(self, adjoint_simulation, sources: Sequence, volume):
        self.adjoint_simulation = adjoint_simulation
        self.sources = list(sources)
        self.volume = volume


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
        return self.terms[0].volume.density

    def forward(self, rho: np.ndarray) -> float:
        """Sets the density of every term's design box, runs the forward
        simulation and evaluates the objective (the adjoint sources are set)."""
        rho = np.asarray(rho, dtype=np.float64)
        for t in self.terms:
            t.volume.density = rho
        self.forward_simulation.run(self.stop, keep=True)
        F = 0.0
        for t in self.terms:
            for s in t.sources:
                F = F + s.eval_functionals_and_set_sources()
        self.value = float(np.real(F))
        self._pending = True
        return self.value

    def gradient(self) -> np.ndarray:
        """dF/drho at the density of the last forward(): one adjoint run per term."""
        if not self._pending:
            raise RuntimeError("gradient() needs a forward() first")
        g = 0
        for t in self.terms:
            t.adjoint_simulation.run(self.stop, keep=True)
            g = g + t.volume.get_sensitivity(exact=self.exact)
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
