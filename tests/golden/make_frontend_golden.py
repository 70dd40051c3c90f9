"""Records the config JSON that the reference's own Python front-end
(ffip/simulation.py, geom.py, source.py) emits for a set of simulations, so
that ffip_gb300's front-end can be checked against it
(tests/test_frontend.py).  Writes tests/golden/frontend.json.

    python tests/golden/make_frontend_golden.py [--ref /path/to/reference]

The reference package imports h5py, shapely and its pybind module, none of
which exist here; they are replaced by empty stand-ins (only JSON building is
exercised).  scipy.integrate.trapz, removed from recent scipy, is aliased to
numpy.trapezoid.
"""
import argparse
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def build_cases(ffip):
    V = ffip.Vector3
    out = {}
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
    out["simulation"] = sim.get_json(ffip.run_until_time(40.0))
    out["stop_dft"] = ffip.run_until_dft(center=V(0, 0, 1), size=V(4, 4, 0), frequency=0.1, field_component="Ez",
                                         time_interval_examined=5, var=1e-3).get_json()
    out["stop_decay"] = ffip.run_until_fields_decay(position=V(1, 0, 0), field_component="Ez", time_interval_examined=3,
                                                    decayed_by=1e-4).get_json()
    ds = {}
    # the reference writes these into input.h5 (Two_Medium_Box.dump, Inhom_Source.dump)
    out["datasets"] = {tmb.dataset_name: tmb.density.ravel().tolist(),
                       "inhom source amplitude a": np.abs(amp.ravel()).tolist(),
                       "inhom source phase a": np.angle(amp.ravel()).tolist()}
    out["epsilon"] = {"m1": [complex(m1.get_epsilon(f)).real for f in (0.05, 0.1, 0.2)] +
                            [complex(m1.get_epsilon(f)).imag for f in (0.05, 0.1, 0.2)],
                      "m1_dis": [complex(m1.get_dis_epsilon(f, 0.25)).real for f in (0.05, 0.1, 0.2)] +
                                [complex(m1.get_dis_epsilon(f, 0.25)).imag for f in (0.05, 0.1, 0.2)]}
    del ds
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FFIP_REFERENCE"), required="FFIP_REFERENCE" not in os.environ,
                    help="reference checkout (default: $FFIP_REFERENCE)")
    a = ap.parse_args()
    for name in ("h5py", "shapely", "shapely.geometry", "ffip._ffip"):
        mod = types.ModuleType(name)
        for attr in ("Point", "LineString", "Polygon", "MultiPolygon", "box"):
            setattr(mod, attr, object)
        sys.modules[name] = mod
    sys.modules["shapely"].geometry = sys.modules["shapely.geometry"]
    import scipy.integrate
    if not hasattr(scipy.integrate, "trapz"):
        scipy.integrate.trapz = np.trapezoid
    sys.path.insert(0, a.ref)
    import ffip
    out = build_cases(ffip)
    with open(os.path.join(HERE, "frontend.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "frontend.json"))


if __name__ == "__main__":
    main()
