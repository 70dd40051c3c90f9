"""Known-answer tests of the time stepper against the physics of a plane
wave at normal incidence on a slab (the reference's check in
scripts/basic tests/plane_wave_fic.py: incident run without the slab, run
with it, flux regions in front of and behind it, R = -(flux of the total
minus the incident fields) / incident flux, T = transmitted / incident flux).

The grid is periodic along x and y (4 x 4 cells), 160 cells long in z with
20-cell CPML at both z faces; an Ex current sheet over the whole period at
z = -50 launches the wave (Gaussian1, f = 0.04); the slab is 20 units thick
between z = -10 - dx/2 and 10 - dx/2 (its faces midway between E nodes);
the flux regions (2 x 2, at z = -30 and +30) read five frequencies in
[0.02, 0.06].  The answers (tests/slab_theory.py):
* the scheme's own reflection and transmission (the 1-D Yee recurrences
  solved through the slab, dispersive nodes with the permittivity that the
  auxiliary-equation update realises): agreement to 1e-4 (absolute, in power
  ratios; measured up to 2e-5, the residue of the CPML and of the finite run);
* lossless slab: R + T = 1 to 1e-4;
* the continuum Airy formula: the error at resolution 2 is at most 0.35 of
  the error at resolution 1 (second-order convergence), at frequencies
  0.01 - 0.03.
The CPU tests run the engine's host emulation; the GPU tests run the CUDA
library (the fused pass with the periodic faces, fp64 and fp32 state)."""
import numpy as np
import pytest

from slab_theory import slab_rt_airy, slab_rt_discrete

FREQS = np.linspace(0.02, 0.06, 5)
TOL = 1e-4


def materials(ffip):
    return {
        "eps4": ffip.Medium(epsilon=4.0),
        "lorentz": ffip.Medium(epsilon=2.0, E_susceptibilities=[
            ffip.LorentzianSusceptibility(frequency=0.05, gamma=0.01, sigma=1.5)]),
        "drude": ffip.Medium(epsilon=1.0, E_susceptibilities=[
            ffip.DrudeSusceptibility(frequency=0.08, gamma=0.01, sigma=1.0)]),
    }


def slab_run(ffip, material, freqs=FREQS, resolution=1, **kw):
    """(R, T) of the stepper, power ratios per frequency."""
    V = ffip.Vector3
    dx = 1.0 / resolution
    period = 4 * dx
    src_f = ffip.Gaussian1(0.04, cutoff=4, start_time=0.0)
    runs = {}
    for tag in ("inc", "tot"):
        src = ffip.Source(function=src_f, center=V(0, 0, -50), size=V(period, period, 0), field_component="Ex")
        geo = [] if tag == "inc" else [ffip.Box(center=V(0, 0, -dx / 2), size=V(3 * period, 3 * period, 20), material=material)]
        sim = ffip.Simulation(size=V(period, period, 160), resolution=resolution, pmls=[ffip.PML(thickness=20, direction="z")],
                              sources=[src], geometry=geo, periodic=[1, 1, 0], **kw)
        r = sim.add_flux_region(center=V(0, 0, -30), size=V(2 * dx, 2 * dx, 0), frequency=freqs)
        t = sim.add_flux_region(center=V(0, 0, 30), size=V(2 * dx, 2 * dx, 0), frequency=freqs)
        sim.run(ffip.run_until_time(800))
        runs[tag] = (r, t)
    inc = runs["inc"][0].get_values()
    refl = runs["tot"][0].get_values(substract=runs["inc"][0])
    trn = runs["tot"][1].get_values()
    return -refl / inc, trn / inc


def discrete_answer(material, freqs=FREQS, resolution=1):
    dx = 1.0 / resolution
    dt = 0.5 * dx
    n = int(round(20 / dx))
    out = [slab_rt_discrete([material.get_dis_epsilon(f, dt)] * n, f, dt, dx) for f in freqs]
    return np.array([o[0] for o in out]), np.array([o[1] for o in out])


def check_discrete(ffip, name, **kw):
    mat = materials(ffip)[name]
    R, T = slab_run(ffip, mat, **kw)
    Rx, Tx = discrete_answer(mat)
    assert np.abs(R - Rx).max() <= TOL, (R, Rx)
    assert np.abs(T - Tx).max() <= TOL, (T, Tx)
    if name == "eps4":
        assert np.abs(R + T - 1).max() <= TOL
        assert Rx.min() > 0.02 and Tx.min() > 0.6  # both waves carry power
    return R, T


@pytest.fixture
def emulated(monkeypatch):
    emu = pytest.importorskip("emu.build_emu")
    from ffip_gb300 import native
    monkeypatch.setattr(native, "_lib", native.load(emu.build()))
    import ffip_gb300 as ffip
    return ffip


@pytest.mark.parametrize("name", ["eps4", "lorentz", "drude"])
def test_emulated_slab_matches_the_discrete_answer(emulated, name):
    check_discrete(emulated, name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["eps4", "lorentz", "drude"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_slab_matches_the_discrete_answer(name, precision):
    import ffip_gb300 as ffip
    from ffip_gb300 import native
    check_discrete(ffip, name, precision=precision, device=0)
    # the periodic faces run in the fused pass
    cfg = ffip.Simulation(size=ffip.Vector3(4, 4, 160), resolution=1, pmls=[ffip.PML(thickness=20, direction="z")],
                          periodic=[1, 1, 0], precision=precision).config(ffip.run_until_time(1))
    with native.NativeSim(cfg) as s:
        assert s.stats()["fused"] == 1


def check_airy_convergence(ffip, **kw):
    """Measured: error 0.016 at resolution 1, 0.0040 at resolution 2."""
    mat = materials(ffip)["eps4"]
    freqs = np.linspace(0.01, 0.03, 5)
    Ra, Ta = slab_rt_airy(4.0, freqs, 20.0)
    err = []
    for res in (1, 2):
        R, T = slab_run(ffip, mat, freqs=freqs, resolution=res, **kw)
        err.append(max(np.abs(R - Ra).max(), np.abs(T - Ta).max()))
    assert 0 < err[0] <= 0.03 and err[1] <= 0.35 * err[0], err


def test_emulated_slab_converges_to_the_airy_formula(emulated):
    check_airy_convergence(emulated)


@pytest.mark.gpu
def test_gpu_slab_converges_to_the_airy_formula():
    import ffip_gb300 as ffip
    check_airy_convergence(ffip, device=0)
