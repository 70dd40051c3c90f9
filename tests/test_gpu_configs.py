"""The plain FP64 vacuum workload exactly as specified, the reference's
sensitivity pipeline on the GPU's own DFT fields, and the failure paths
(divergence check, bounded device waits), through the C ABI on the GPU.

Tolerances (relative to the largest |DFT| of the monitor group):
  fp64 state:  1e-10  (the drop-in bar)
  fp32 state:  1e-4   (fp32 fields, fp64 DFT sums)
"""
import copy

import numpy as np
import pytest
from scipy.interpolate import RegularGridInterpolator

from golden_cases import flatten, load
from test_gpu_adjoint import interpn_transpose_ref

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4


def rel_err(out, ref):
    worst = 0.0
    for k, r in ref.items():
        assert out[k].shape == r.shape, k
        if k.endswith("/real") or k.endswith("/imag"):
            g = k.rsplit("/", 1)[0]
            scale = max(np.abs(ref[g + "/real"]).max(), np.abs(ref[g + "/imag"]).max())
            assert scale > 0, g
            worst = max(worst, np.abs(out[k] - r).max() / scale)
        else:
            assert np.array_equal(out[k], r), k
    return worst


@pytest.fixture(scope="module")
def vacuum64_oracle():
    """The plain vacuum workload on the oracle (the reference's loops
    restated): 64^3 cells, 8-cell CPML (order 3, R = 1e-8), one Ez point
    current at a seeded interior cell, Gaussian1 at f = 0.1, 1000 steps, an Ez
    DFT plane at z = 48 cells (z = +16) at 0.08, 0.1 and 0.12."""
    from ffip_gb300 import workloads
    from oracle import port
    cfg = workloads.vacuum_point(64, steps=1000, precision="fp64")
    return cfg, flatten(port.run_json(cfg, {}, threads=8))


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32", FP32_TOL)])
def test_vacuum64_point_source_matches_oracle(vacuum64_oracle, precision, tol):
    from ffip_gb300 import native
    cfg, ref = vacuum64_oracle
    c = copy.deepcopy(cfg)
    c["precision"] = precision
    c["device"] = 0
    with native.NativeSim(c) as s:
        assert s.stats()["fused"] == 1
        s.run(c["stop condition"])
        assert s.stats()["time_step"] == 1000
        out = flatten(s.outputs())
    g = "volume fields dft 0"
    assert out[g + "/real"].shape == (3, 2, 65, 65)  # the Ez plane's closure: two z planes
    assert rel_err(out, ref) <= tol


# ---------------------------------------------------------------------------
# Adjoint_Volume.get_sensitivity (ffip/simulation.py:841-869) and
# _ffip.transpose (app/ffip.cpp:308-352), restated with numpy / scipy, on the
# DFT fields of a forward and an adjoint run of the GPU stepper


def reference_dft_interpolant(group, dx):
    """Fields_DFT.read + get_interpolant of the reference
    (ffip/simulation.py:55-91): size-1 axes widened by +-dx/2 (frequency by
    0.9 / 1.1) with the values repeated, then linear interpolation over
    (f, z, y, x)."""
    f, x, y, z = (np.asarray(group[k], dtype=float) for k in ("f", "x", "y", "z"))
    v = group["real"] + 1j * group["imag"]
    if f.size == 1:
        f = f * np.array([0.9, 1.1])
    if x.size == 1:
        x = x + np.array([-dx / 2, dx / 2])
    if y.size == 1:
        y = y + np.array([-dx / 2, dx / 2])
    if z.size == 1:
        z = z + np.array([-dx / 2, dx / 2])
    for i in range(4):
        if v.shape[i] == 1:
            v = np.concatenate((v, v), axis=i)
    return RegularGridInterpolator((f, z, y, x), v, method="linear", bounds_error=True)


def reference_sensitivity(vol, fwd_out, adj_out, points, dx):
    """se_i = Re(2 pi j f E_fwd,i E_adj,i eps'(rho_i) / norm) at the points of
    each E component, scattered onto the density nodes with the transposed
    trilinear weights, summed over the three components."""
    rho_interp = RegularGridInterpolator((vol.z, vol.y, vol.x), vol.density, bounds_error=True)
    res = 0
    for i in range(3):
        x, y, z = points[i]
        pts = np.stack((vol.frequency * np.ones(z.shape), z, y, x), axis=-1)
        ef = reference_dft_interpolant(fwd_out[vol.forward_dfts[i].group_name], dx)(pts)
        ea = reference_dft_interpolant(adj_out[vol.adjoint_dfts[i].group_name], dx)(pts)
        rho = rho_interp(np.stack((z, y, x), axis=-1))
        se = np.real(2j * np.pi * vol.frequency * ef * ea * vol.epsilon_der(rho) / vol.norm)
        res = res + interpn_transpose_ref(vol.x, vol.y, vol.z, np.stack((x, y, z, se), axis=-1))
    return np.reshape(res, vol.shape)


def test_reference_sensitivity_pipeline_on_gpu_dft_fields():
    """The GPU correlation + transpose (ffip_sensitivity with w = 2 pi j f)
    equals the reference's pipeline restated in numpy, on the same DFT
    fields: at the exact coordinates of the design box's E points (what the
    rebuild uses) and at the geometry-info coordinates the simulation
    reports (the reference's own points, truncated to integers by
    src/simulation.cpp:200-211)."""
    import ffip_gb300 as ffip
    from ffip_gb300.simulation import frequency_factor, sensitivity_scatter
    V = ffip.Vector3
    f0 = 0.1
    pml = [ffip.PML(thickness=6, sigma_max=6.14)]
    fwd = ffip.Simulation(size=V(24, 24, 24), resolution=1, pmls=pml, precision="fp64", device=0,
                          sources=[ffip.Source(function=ffip.Gaussian1(f0, cutoff=4, start_time=0.0),
                                               center=V(0, 0, -6), size=V(12, 12, 0), field_component="Ex")])
    adj = ffip.Simulation(size=V(24, 24, 24), resolution=1, pmls=pml, precision="fp64", device=0)
    asrc = ffip.Adjoint_Source(adj, fwd, function=ffip.Gaussian1(f0, cutoff=4, start_time=5.0), frequency=f0,
                               center=V(0.5, 0, 5), size=V(2, 2, 0), dim=V(2, 2, 1),
                               udfs=[ffip.field_match_objective(np.zeros((1, 2, 2)), "Ex", weight=2.0)])
    rho = np.random.default_rng(1).uniform(0.3, 0.7, size=(4, 5, 5))
    vol = ffip.Adjoint_Volume(adj, fwd, frequency=f0, center=V(0, 0, 0), size=V(8, 8, 6), dim=V(5, 5, 4), density=rho,
                              medium1=ffip.Medium(epsilon=3), medium2=ffip.Medium(), norm=0.7 - 0.4j)
    stop = ffip.run_until_time(300)
    fwd.run(stop)
    asrc.eval_functionals_and_set_sources()  # the adjoint sources from the forward fields
    adj.run(stop)
    dx = fwd.dx
    exact_pts = [vol.design_points(i) for i in range(3)]
    got = vol.get_sensitivity(exact=False)
    want = reference_sensitivity(vol, fwd.outputs, adj.outputs, exact_pts, dx)
    assert np.abs(want).max() > 0
    assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max()
    # the reference's own points: the geometry-info coordinates
    gi_pts = [(vol.geom_infos[i].x, vol.geom_infos[i].y, vol.geom_infos[i].z) for i in range(3)]
    want_gi = reference_sensitivity(vol, fwd.outputs, adj.outputs, gi_pts, dx)
    rho_interp = RegularGridInterpolator((vol.z, vol.y, vol.x), vol.density, bounds_error=True)
    got_gi = 0
    for i in range(3):
        x, y, z = gi_pts[i]
        pts = np.stack((f0 * np.ones(z.shape), z, y, x), axis=-1)
        ef = vol.forward_dfts[i].get_interpolant(method="linear", bounds_error=True)(pts)
        ea = vol.adjoint_dfts[i].get_interpolant(method="linear", bounds_error=True)(pts)
        deps = vol.epsilon_der(rho_interp(np.stack((z, y, x), axis=-1)))
        got_gi = got_gi + sensitivity_scatter(frequency_factor(f0), vol.norm, ef, ea, np.asarray(deps, dtype=complex),
                                              x, y, z, vol.x, vol.y, vol.z)
    got_gi = np.reshape(got_gi, vol.shape)
    assert np.abs(want_gi).max() > 0
    assert np.abs(got_gi - want_gi).max() <= 1e-10 * np.abs(want_gi).max()
    fwd.release()
    adj.release()


# ---------------------------------------------------------------------------
# failure paths: no GPU fault is involved (a host-side check of the field
# values, and a device wait on a barrier that nothing completes)


@pytest.mark.parametrize("precision,steps", [("fp32", 200), ("fp64", 1300)])
def test_divergence_check_stops_the_unstable_debye_run(precision, steps):
    """The reference's Debye pole (b2 = 0) is unconditionally unstable; run
    long, its fields overflow.  With a check every 100 steps the fused GPU
    stepper stops with FFIP_ERR_DIVERGED at the first check that sees them,
    and with the check off it runs on."""
    from ffip_gb300 import native
    cfg, ds, _ = load("debye_short")
    cfg = copy.deepcopy(cfg)
    cfg["precision"] = precision
    cfg["device"] = 0
    cfg["divergence check interval"] = 100
    with native.NativeSim(cfg, ds) as s:
        assert s.stats()["fused"] == 1
        with pytest.raises(native.FfipError, match=r"error -5: the simulation diverged"):
            s.step(3000)
        # the same check as the emulated engine's (identical arithmetic)
        assert abs(s.stats()["time_step"] - steps) <= 100
    cfg["divergence check interval"] = 0
    with native.NativeSim(cfg, ds) as s:
        s.step(steps + 100)
        out = flatten(s.outputs())
        assert not all(np.isfinite(v).all() for k, v in out.items() if k.endswith("/real"))


def test_fused_wait_timeout_is_reported_and_the_context_survives():
    """"fused wait test" makes every CTA of the fused pass wait on a barrier
    that nothing completes; with a 2 ms bound the waits give up, the CTAs
    drain their TMA copies and leave, and the next synchronising call
    returns FFIP_ERR_CUDA with the timeout message.  The handle is then
    destroyed, and a new handle on the same device gives the golden result."""
    from ffip_gb300 import native
    lib = native.load()
    cfg, ds, ref = load("vacuum_pml")
    bad = copy.deepcopy(cfg)
    bad.update({"device": 0, "fused wait test": True, "fused wait timeout": 0.002})
    s = native.NativeSim(bad, ds)
    try:
        assert s.stats()["fused"] == 1
        s.step(3)
        rc = lib.ffip_sync(s.h)
        assert rc == -2
        assert "timed out" in lib.ffip_last_error().decode()
        # reported until the state is reset
        assert lib.ffip_sync(s.h) == -2
        assert lib.ffip_reset(s.h) == 0
        assert lib.ffip_sync(s.h) == 0
    finally:
        s.close()
    good = copy.deepcopy(cfg)
    good["device"] = 0
    assert rel_err(flatten(native.run_json(good, ds)), ref) <= FP64_TOL
