"""Material rasterisation on the GPU (raster.cu) against the host's
restatement of the reference's set_materials_from_geometry (plan.cpp
rasterize_media): the device tables (slot map, row ranges, g_inf, dt/g_inf,
1/g_inf, pole groups, packed records, amplitudes) hash to the same values,
and the runs give bit-identical DFT outputs, on every golden case, the
dispersive-spheres workload at full size, and the adjoint-design forward
simulation before and after a density update."""
import copy

import numpy as np
import pytest

from golden_cases import CASES, flatten, load

pytestmark = pytest.mark.gpu


def make(cfg, ds, rasterize, precision=None):
    from ffip_gb300 import native
    c = copy.deepcopy(cfg)
    c["rasterize"] = rasterize
    c["device"] = 0
    if precision:
        c["precision"] = precision
    return native.NativeSim(c, ds)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_golden_case_tables_and_outputs_equal_the_host_rasterisation(name, precision):
    cfg, ds, _ = load(name)
    outs, sums = {}, {}
    for r in ("host", "device"):
        with make(cfg, ds, r, precision) as s:
            cs, dev = s.media_info()
            assert dev == (r == "device")
            sums[r] = cs
            s.run(cfg["stop condition"])
            outs[r] = flatten(s.outputs())
    assert sums["host"] == sums["device"]
    for k in outs["host"]:
        assert np.array_equal(outs["host"][k], outs["device"][k]), k


def test_auto_rasterises_on_the_gpu():
    cfg, ds, _ = load("dispersive")
    with make(cfg, ds, "auto") as s:
        assert s.media_info()[1]


def test_dispersive_spheres_256_tables_equal_the_host_rasterisation():
    from ffip_gb300 import workloads
    cfg = workloads.dispersive_spheres(256, precision="fp32")
    sums = {}
    for r in ("host", "device"):
        with make(cfg, {}, r) as s:
            sums[r] = s.media_info()[0]
    assert sums["host"] == sums["device"]


def adjoint_forward_config():
    """The adjoint-design workload's forward simulation (192 x 192 x 160
    cells, 96 x 96 x 24 two-medium design box, eps = 1 + 11 rho)."""
    from ffip_gb300 import workloads
    prob, rho = workloads.adjoint_design(precision="fp32")
    sim = prob.forward_simulation
    cfg = sim.config(prob.stop)
    ds = sim.dump()
    name = [k for k in ds if k.startswith("two medium box")][0]
    return cfg, ds, name, rho


def test_adjoint_design_density_update_equals_the_host_rasterisation():
    cfg, ds, name, rho = adjoint_forward_config()
    rho2 = np.clip(rho + 0.2 * np.random.default_rng(3).normal(size=rho.shape), 0, 1)
    sums = {}
    for r in ("host", "device"):
        with make(cfg, ds, r) as s:
            first = s.media_info()[0]
            s.set_density(name, rho2)
            sums[r] = (first, s.media_info()[0])
    assert sums["host"] == sums["device"]
    assert sums["host"][0] != sums["host"][1]


def test_density_box_with_more_candidate_poles_falls_back_to_the_host():
    """A general medium box whose medium table uses more distinct poles (13)
    than the device rasterisation's candidate list holds (12) -- each table
    entry two of them, so a point has at most four -- is rasterised on the
    host under "auto", with the same outputs as "host", and "device" refuses
    it with a clear error."""
    from ffip_gb300 import native
    cfg, ds, _ = load("density_boxes")
    cfg, ds = copy.deepcopy(cfg), dict(ds)
    box = [g for g in cfg["geometry"] if g["type"] == "general medium box"][0]
    npole, nfun = 13, len(ds[box["density function dataset"]])
    box["medium"]["electric susceptibility"] = [
        {"type": "Lorentz", "frequency": 0.1 + 0.01 * t, "gamma": 0.02, "amplitude": 1.0} for t in range(npole)]
    amp = np.zeros((nfun, npole))
    for i in range(nfun):
        amp[i, i % npole] = 0.5
        amp[i, (i + 2) % npole] = 0.25
    ds[box["electric susceptibility amplitudes dataset"]] = amp.ravel()
    outs = {}
    for r in ("auto", "host"):
        with make(cfg, ds, r, "fp64") as s:
            assert not s.media_info()[1]
            s.run(cfg["stop condition"])
            outs[r] = flatten(s.outputs())
    for k in outs["host"]:
        assert np.array_equal(outs["host"][k], outs["auto"][k]), k
    with pytest.raises(native.FfipError, match="device rasterisation"):
        make(cfg, ds, "device", "fp64")
