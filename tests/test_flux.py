"""Flux regions / boxes and Adjoint_Flux against numpy restatements of the
reference (ffip/simulation.py:94-251 Flux_Region / Flux_Box, 585-645
Adjoint_Flux), on the engine's host emulation (no GPU): the front-end's
numpy flux, the device-reduction path (ffip_flux, run here by the emulated
backend with the same per-point rules) and the adjoint source amplitudes."""
import numpy as np
import pytest
from scipy.interpolate import RegularGridInterpolator

emu = pytest.importorskip("emu.build_emu")


@pytest.fixture
def emulated(monkeypatch):
    from ffip_gb300 import native
    monkeypatch.setattr(native, "_lib", native.load(emu.build()))
    return native


def reference_interpolant(group, dx):
    """Fields_DFT.read + get_interpolant (ffip/simulation.py:55-91)."""
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


def reference_flux(outputs, e1_group, h2_group, center, size, freqs, weight, dx, scale=1):
    """Flux_Region.get_values (ffip/simulation.py:121-160): trapezoid weights
    on a grid of round(size / dx * scale) + 1 points per axis."""
    n = [int(round(s / dx * scale)) + 1 for s in size]
    p1 = [c - s / 2 for c, s in zip(center, size)]
    p2 = [c + s / 2 for c, s in zip(center, size)]
    ax = [np.linspace(p1[a], p2[a], n[a]) for a in range(3)]
    pts = np.stack(np.meshgrid(np.sort(freqs), ax[2], ax[1], ax[0], indexing="ij"), axis=-1)
    e1 = reference_interpolant(outputs[e1_group], dx)(pts)
    h2 = reference_interpolant(outputs[h2_group], dx)(pts)
    meas = 1.0
    ws = []
    for a in range(3):
        w = np.ones(n[a])
        if n[a] > 1:
            meas *= size[a] / (n[a] - 1)
            w[0] = w[-1] = 0.5
        ws.append(w)
    Z, Y, X = np.meshgrid(ws[2], ws[1], ws[0], indexing="ij")
    wts = X * Y * Z * meas * weight
    return np.sum(np.real(e1 * np.conj(h2)) * wts, axis=(1, 2, 3)), e1, h2, wts


def small_simulation(ffip, freqs):
    V = ffip.Vector3
    src = ffip.Source(function=ffip.Gaussian1(0.1, cutoff=4, start_time=0.0), center=V(0.5, 0, -2), size=V(4, 4, 0),
                      field_component="Ex")
    sim = ffip.Simulation(size=V(16, 16, 16), resolution=1, pmls=[ffip.PML(thickness=4, sigma_max=4.0)], sources=[src])
    box = sim.add_flux_box(center=V(0, 0, 0), size=V(6, 6, 6), frequency=freqs)
    plane = sim.add_flux_region(center=V(0, 0, 3), size=V(6, 4, 0), frequency=freqs, weight=1)
    return sim, box, plane


def check_flux(ffip, sim, box, plane, freqs):
    """Front-end and device flux of the plane (scales 1 and 2) and the box
    against the reference restatement."""
    for scale in (1, 2):
        want, *_ = reference_flux(sim.outputs, plane.e1_dft.group_name, plane.h2_dft.group_name, [0, 0, 3], [6, 4, 0],
                                  freqs, 1, sim.dx, scale)
        got = plane.get_values(scale=scale)
        dev = plane.get_values(scale=scale, device=True)
        assert np.abs(want).max() > 0
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
        np.testing.assert_allclose(dev, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    # the box: six outward-weighted planes
    want = 0
    for r in box.flux_regions:
        w, *_ = reference_flux(sim.outputs, r.e1_dft.group_name, r.h2_dft.group_name, r.center.get_json(),
                               r.size.get_json(), freqs, float(r.weight), sim.dx)
        want = want + w
    np.testing.assert_allclose(box.get_values(), want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    np.testing.assert_allclose(box.get_values(device=True), want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_flux_regions_match_the_reference_restatement_and_the_device_sum(emulated):
    import ffip_gb300 as ffip
    freqs = [0.08, 0.1, 0.12]
    sim, box, plane = small_simulation(ffip, freqs)
    sim.run(ffip.run_until_time(120), keep=True)
    try:
        check_flux(ffip, sim, box, plane, freqs)
    finally:
        sim.release()


def test_device_flux_needs_a_kept_simulation_and_registered_frequencies(emulated):
    import ffip_gb300 as ffip
    sim, box, plane = small_simulation(ffip, [0.1])
    sim.run(ffip.run_until_time(20))
    with pytest.raises(RuntimeError, match="kept"):
        plane.get_values(device=True)
    sim.run(ffip.run_until_time(20), keep=True)
    try:
        kept = sim._kept["sim"]
        with pytest.raises(ffip.FfipError, match="not registered"):
            kept.flux(plane.e1_dft.group_name, plane.h2_dft.group_name, [0.0], [0.0], [3.0], [1.0], [0.2])
        with pytest.raises(ffip.FfipError, match="no monitor group"):
            kept.flux("nope", plane.h2_dft.group_name, [0.0], [0.0], [3.0], [1.0], [0.1])
    finally:
        sim.release()


def test_adjoint_flux_sources_match_the_reference_restatement(emulated):
    """Adjoint_Flux.eval_functionals_and_set_sources (ffip/simulation.py:
    632-645): the objective is the region's flux, the electric adjoint
    source amplitude conj(H2) w and the magnetic one -conj(E1) w on the
    integration grid."""
    import ffip_gb300 as ffip
    V = ffip.Vector3
    fwd, box, plane = small_simulation(ffip, [0.1])
    adj = ffip.Simulation(size=V(16, 16, 16), resolution=1, pmls=[ffip.PML(thickness=4, sigma_max=4.0)])
    af = ffip.Adjoint_Flux(adj, fwd, ffip.Gaussian1(0.1, cutoff=4, start_time=5.0), fluxes=[plane], frequency=0.1, scale=2)
    fwd.run(ffip.run_until_time(120))
    F = af.eval_functionals_and_set_sources()
    want, e1, h2, w = reference_flux(fwd.outputs, plane.e1_dft.group_name, plane.h2_dft.group_name, [0, 0, 3], [6, 4, 0],
                                     [0.1], 1, fwd.dx, scale=2)
    np.testing.assert_allclose(F, want, rtol=1e-12)
    np.testing.assert_allclose(af.e_adjoint_sources[0].amplitude, np.conj(h2[0]) * w, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(af.m_adjoint_sources[0].amplitude, -np.conj(e1[0]) * w, rtol=1e-12, atol=1e-15)
    assert af.e_adjoint_sources[0].field_component == "Ex" and af.m_adjoint_sources[0].field_component == "Hy"
    # the integration grid at scale 2: 13 x 9 points on the z plane
    assert af.e_adjoint_sources[0].shape == (1, 9, 13)
