"""The Python front-end emits the same config JSON and input datasets as the
reference's own ffip/simulation.py, geom.py and source.py for the same
objects (fixture: tests/golden/frontend.json, generated by
tests/golden/make_frontend_golden.py from the reference's code)."""
import json
import os

import numpy as np

import ffip_gb300 as ffip

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "frontend.json")


def build():
    V = ffip.Vector3
    lor = ffip.LorentzianSusceptibility(frequency=0.12, gamma=0.01, sigma=1.5)
    dru = ffip.DrudeSusceptibility(frequency=0.3, gamma=0.02, sigma=0.8)
    deb = ffip.DeybeSusceptibility(tau=2.0, sigma=0.4)
    m1 = ffip.Medium(epsilon=2.0, E_susceptibilities=[lor, dru])
    m2 = ffip.Medium(epsilon=1.5, mu=1.2, E_conductivity=0.05, M_conductivity=0.01, E_susceptibilities=[deb])
    src = ffip.Source(function=ffip.Gaussian1(0.1, cutoff=4, start_time=1.0), center=V(0.5, -0.5, -3), size=V(4, 4, 0),
                      amplitude=2.0, field_component="Ey")
    pmls = [ffip.PML(thickness=3), ffip.PML(thickness=2, direction="z", side="positive", k_max=2, order=2)]
    sim = ffip.Simulation(size=V(16, 16, 16), resolution=2, pmls=pmls, sources=[src], default_material=ffip.Medium(),
                          progress_interval=10, courant=0.4, input_file="in.h5", fields_output_file="out.h5")
    sim.add_geometry(ffip.Sphere(2.5, material=m1, center=V(1, 0, 0)))
    sim.add_geometry(ffip.Box(size=V(3, 2, 1), material=m2, center=V(-2, 1, 2)))
    rho = np.linspace(0, 1, 3 * 4 * 5).reshape(3, 4, 5)
    tmb = ffip.Two_Medium_Box(size=V(4, 3, 2), center=V(0, 0, 3), dim=V(5, 4, 3), density=rho,
                              medium1=ffip.Medium(epsilon=12), medium2=ffip.Medium(), suffix="1")
    sim.add_geometry(tmb)
    amp = (np.arange(6) + 1.0).reshape(1, 2, 3) * np.exp(1j * np.arange(6).reshape(1, 2, 3))
    sim.add_source(ffip.Inhom_Source(function=ffip.Gaussian1(0.12), amplitude=amp, frequency=0.12, center=V(0, 0, -2),
                                     size=V(2, 1, 0), dim=V(3, 2, 1), field_component="Ex", suffix="a"))
    sim.add_dft_fields(center=V(0, 0, 1), size=V(4, 4, 0), frequency=[0.12, 0.1], field_component="Ez")
    sim.add_dft_fields(center=V(1, 1, 1), size=V(2, 2, 2), frequency=[0.1], field_component="Hx")
    sim.add_flux_region(center=V(0, 0, 4), size=V(4, 4, 0), frequency=[0.1], weight=1)
    sim.request_geom_info(tmb, field_component="Ey")
    return sim, m1, tmb


def test_simulation_json_matches_reference():
    gold = json.load(open(GOLD))
    sim, _, _ = build()
    mine = json.loads(json.dumps(sim.get_json(ffip.run_until_time(40.0))))
    assert mine == gold["simulation"]


def test_stop_conditions_match_reference():
    gold = json.load(open(GOLD))
    V = ffip.Vector3
    assert ffip.run_until_dft(center=V(0, 0, 1), size=V(4, 4, 0), frequency=0.1, field_component="Ez",
                              time_interval_examined=5, var=1e-3).get_json() == gold["stop_dft"]
    assert ffip.run_until_fields_decay(position=V(1, 0, 0), field_component="Ez", time_interval_examined=3,
                                       decayed_by=1e-4).get_json() == gold["stop_decay"]


def test_datasets_match_reference():
    gold = json.load(open(GOLD))
    sim, _, _ = build()
    ds = sim.dump()
    assert sorted(ds) == sorted(gold["datasets"])
    for k, v in gold["datasets"].items():
        np.testing.assert_array_equal(np.asarray(ds[k]), np.asarray(v))


def test_medium_epsilon_matches_reference():
    gold = json.load(open(GOLD))
    _, m1, _ = build()
    e = [complex(m1.get_epsilon(f)) for f in (0.05, 0.1, 0.2)]
    d = [complex(m1.get_dis_epsilon(f, 0.25)) for f in (0.05, 0.1, 0.2)]
    np.testing.assert_allclose([c.real for c in e] + [c.imag for c in e], gold["epsilon"]["m1"], rtol=1e-14)
    np.testing.assert_allclose([c.real for c in d] + [c.imag for c in d], gold["epsilon"]["m1_dis"], rtol=1e-14)


def test_pml_keeps_explicit_sigma_max():
    p = ffip.PML(thickness=2, sigma_max=3.0)
    ffip.Simulation(size=ffip.Vector3(8, 8, 8), resolution=1, pmls=[p])
    assert p.get_json()["sigma max"] == 3.0


def test_dft_values_at_grid_nodes_read_directly_equal_the_interpolant():
    """Adjoint_Volume reads the forward / adjoint DFT monitors at the design
    box's own grid points: directly where the points are nodes of the
    monitor's output grid, through the reference's linear interpolant
    (ffip/simulation.py:55-91) elsewhere; at the nodes the two agree to
    rounding (the interpolant's weights at a node are 0 and 1 up to an ulp;
    the widened one-frequency axis averages two equal values)."""
    from ffip_gb300.geom import Vector3
    from ffip_gb300.simulation import Fields_DFT, _dft_at_points
    rng = np.random.default_rng(0)
    d = Fields_DFT(Vector3(0, 0, 0), Vector3(4, 3, 0), [0.1], "Ex", suffix="t", dx=1.0)
    x, y, z = np.arange(-2.5, 2.6, 1.0), np.arange(-1.5, 1.6, 0.5), np.array([0.0])
    shape = (1, z.size, y.size, x.size)
    d.read({d.group_name: {"f": np.array([0.1]), "x": x, "y": y, "z": z, "real": rng.normal(size=shape),
                           "imag": rng.normal(size=shape)}})
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    got = _dft_at_points(d, 0.1, X.ravel(), Y.ravel(), Z.ravel())
    want = d.get_interpolant(method="linear", bounds_error=True)(
        np.stack((np.full(X.size, 0.1), Z.ravel(), Y.ravel(), X.ravel()), axis=-1))
    np.testing.assert_allclose(got, want, rtol=1e-14, atol=1e-15)
    # off-node points take the interpolant
    xs = np.array([-2.0, 0.25]), np.array([-1.5, 0.0]), np.array([0.0, 0.0])
    off = _dft_at_points(d, 0.1, *xs)
    np.testing.assert_allclose(off, d.get_interpolant(method="linear")(np.stack((np.full(2, 0.1), xs[2], xs[1], xs[0]), -1)))
