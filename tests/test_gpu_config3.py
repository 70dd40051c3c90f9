"""Adjoint gradient of the adjoint-design workload at its full size, against
central finite differences, on the GPU stepper.

Workload (ffip_gb300.workloads.adjoint_design): 192 x 192 x 160 cells,
16-cell CPML, a 96 x 96 x 24 design box (97 x 97 x 25 density nodes of
seeded filtered noise, eps = 1 + 11 rho), an Ex current sheet below it,
objective F = sum of |Ex|^2 at 4 seeded probe cells above it at 0.09, 0.1 and
0.11; every run 5000 steps.  The gradient (one forward run, the adjoint
run(s), the GPU correlation and transpose) is compared with central
differences (h = 1e-3) of F at 16 seeded density nodes, the differences
taken with fp64 state (fp32 state rounds F at about 1e-7 of its value, which
h = 1e-3 turns into noise far above the gradient).  Bound: 1e-3 relative
per node, for the fp64-state and the fp32-state gradient.  The gradient
comes from one broadband adjoint run for the three frequencies
(design.BroadbandAdjoint); with fp64 state it also equals the sum of three
per-frequency adjoint runs (the reference's scheme) to 1e-3."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-3
NODES = 16


@pytest.fixture(scope="module")
def nodes():
    from ffip_gb300 import workloads
    _, rho0 = workloads.adjoint_design(precision="fp64")
    rng = np.random.default_rng(16)
    # interior nodes of the design box (z, y, x)
    nz, ny, nx = rho0.shape
    return [(int(rng.integers(1, nz - 1)), int(rng.integers(1, ny - 1)), int(rng.integers(1, nx - 1))) for _ in range(NODES)]


@pytest.fixture(scope="module")
def fd(nodes):
    from ffip_gb300 import workloads
    prob, rho0 = workloads.adjoint_design(precision="fp64")
    for s in [prob.forward_simulation] + [t.adjoint_simulation for t in prob.terms]:
        s.device = 0
    out = {}
    try:
        F0 = prob.forward(rho0)
        for n in nodes:
            Fs = []
            for sgn in (1, -1):
                r = rho0.copy()
                r[n] += sgn * H
                Fs.append(prob.forward(r))
            out[n] = (Fs[0] - Fs[1]) / (2 * H)
    finally:
        prob.release()
    return F0, out


@pytest.fixture(scope="module")
def grads():
    from ffip_gb300 import workloads
    res = {}
    for precision, broadband in (("fp64", True), ("fp32", True), ("fp64 per frequency", False)):
        prob, rho0 = workloads.adjoint_design(precision=precision.split()[0], broadband=broadband)
        assert len(prob.terms) == (1 if broadband else 3)
        for s in [prob.forward_simulation] + [t.adjoint_simulation for t in prob.terms]:
            s.device = 0
        try:
            res[precision] = prob.value_and_gradient(rho0)
        finally:
            prob.release()
    return res


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_full_size_gradient_matches_central_differences(fd, grads, nodes, precision):
    F0, d = fd
    F, g = grads[precision]
    assert abs(F - F0) <= (1e-12 if precision == "fp64" else 1e-4) * abs(F0)
    errs = {n: abs(g[n] - d[n]) / abs(d[n]) for n in nodes}
    assert max(errs.values()) <= 1e-3, errs


def test_broadband_adjoint_equals_the_per_frequency_runs(grads):
    F1, g1 = grads["fp64"]
    F3, g3 = grads["fp64 per frequency"]
    assert abs(F1 - F3) <= 1e-14 * abs(F3)
    assert np.abs(g1 - g3).max() <= 1e-3 * np.abs(g3).max()
