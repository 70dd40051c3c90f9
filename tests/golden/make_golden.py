"""Generates the golden fixtures in tests/golden/ by running the reference's
own FDTD code (compiled from its sources by oracle/Makefile.ref into
oracle/_ref/run_sim_json) on small seeded configurations.

Each case is written to <case>.json (config + input datasets) and
<case>.npz (every output dataset the reference wrote, keyed "group/name").

    python tests/golden/make_golden.py [--ref /path/to/reference]

Needs the reference checkout (only in the build container); the fixtures it
writes are what the tests use everywhere else.
"""
import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def medium(eps=1.0, mu=1.0, econd=0.0, mcond=0.0, esus=(), msus=()):
    return {"epsilon": eps, "mu": mu, "electric conductivity": econd, "magnetic conductivity": mcond,
            "electric susceptibility": list(esus), "magnetic susceptibility": list(msus)}


def lorentz(f, g, a):
    return {"type": "Lorentz", "frequency": f, "gamma": g, "amplitude": a}


def drude(f, g, a):
    return {"type": "Drude", "frequency": f, "gamma": g, "amplitude": a}


def debye(tau, a):
    return {"type": "Deybe", "tau": tau, "amplitude": a}


def gauss1(f, cutoff=4.0, st=0.0):
    return {"type": "Gaussian1", "frequency": f, "cutoff": cutoff, "start time": st}


def vsrc(center, size, comp, f, amp=1.0, st=0.0):
    return {"type": "volume source", "center": center, "size": size, "amplitude": amp,
            "field component": comp, "function": gauss1(f, 4.0, st)}


def dft(center, size, comp, freqs, k):
    return {"type": "volume fields dft", "center": center, "size": size, "frequency": freqs,
            "field component": comp, "output group": "volume fields dft %d" % k}


def pml(th, smax, kmax=1.0, order=3, **kw):
    d = {"thickness": th, "k max": kmax, "sigma max": smax, "order": order}
    d.update(kw)
    return d


def base(size, res=1.0, sc=0.5):
    return {"courant number": sc, "resolution": res, "size": size, "input file": "input.h5",
            "fields output file": "output.h5", "default material": medium(), "progress interval": 1000}


def cases():
    rng = np.random.default_rng(20241203)
    out = {}

    # 1. vacuum + CPML on all faces, Ez point source off-grid, E and H monitors
    c = base([16, 16, 16])
    c["PML"] = [pml(4, 3.45)]
    c["sources"] = [vsrc([0.3, -0.6, 0.25], [0, 0, 0], "Ez", 0.1)]
    c["fields output"] = [dft([0, 0, 3], [6, 6, 0], "Ez", [0.08, 0.1, 0.12], 0),
                          dft([1, 0, -1], [4, 5, 3], "Hx", [0.1, 0.09], 1),
                          dft([0, 0, 3], [6, 6, 0], "Ez", [0.1], 2)]
    c["stop condition"] = {"type": "time", "time": 60}
    out["vacuum_pml"] = (c, {})

    # 2. dispersive spheres (2-pole Lorentz, Drude), a conductive box, a
    #    Debye box; Ex sheet source; E, D volume monitors; geometry info
    c = base([20, 20, 20])
    c["PML"] = [pml(4, 3.45)]
    lor = medium(2.0, esus=[lorentz(0.12, 0.01, 1.5), lorentz(0.18, 0.02, 0.7)])
    dru = medium(1.0, esus=[drude(0.25, 0.03, 1.0)])
    c["geometry"] = [
        {"type": "sphere", "center": [-2.3, 1.1, 0.4], "radius": 3.2, "medium": lor},
        {"type": "sphere", "center": [2.6, -1.7, 1.0], "radius": 2.6, "medium": dru},
        {"type": "box", "center": [0.5, 3.5, -3.0], "size": [5, 2, 3], "medium": medium(3.0, econd=0.05)},
    ]
    c["sources"] = [vsrc([0, 0, -4.5], [8, 8, 0], "Ex", 0.11)]
    c["fields output"] = [dft([0, 0, 0.5], [8, 8, 4], "Ex", [0.09, 0.11, 0.13], 0),
                          dft([0, 0, 0.5], [8, 8, 4], "Dx", [0.11], 1),
                          dft([0, 0, 2], [6, 6, 0], "Ey", [0.11], 2)]
    c["geometry info request"] = [{"field component": "Ex", "geometry index": 0, "output group": "geometry info request 0 Ex"}]
    c["stop condition"] = {"type": "time", "time": 80}
    out["dispersive"] = (c, {})

    # 2b. Debye medium.  The reference's discretisation of a Debye pole
    #     (b2 = 0 in src/medium.cpp:24-31) has a root of modulus > 1, so the
    #     field grows without bound; a short run still pins the update rule.
    c = base([12, 12, 12])
    c["PML"] = [pml(3, 4.6)]
    c["geometry"] = [{"type": "box", "center": [0.5, 0, 0], "size": [4, 4, 4], "medium": medium(1.5, esus=[debye(2.0, 1.2)])}]
    c["sources"] = [vsrc([-2.0, 0.5, 0.0], [0, 0, 0], "Ey", 0.12)]
    c["fields output"] = [dft([0, 0, 0], [6, 6, 6], "Ey", [0.1, 0.12], 0)]
    c["stop condition"] = {"type": "time", "time": 20}
    out["debye_short"] = (c, {})

    # 3. two-medium box with a density dataset, general medium box with
    #    tabulated pole amplitudes, inhomogeneous source with amp/phase
    c = base([16, 16, 16])
    c["PML"] = [pml(3, 4.6)]
    dim = [5, 4, 3]
    rho = rng.uniform(0, 1, size=(dim[2], dim[1], dim[0]))
    gdim = [4, 3, 3]
    grho = rng.uniform(0, 1, size=(gdim[2], gdim[1], gdim[0]))
    rf = np.linspace(0, 1, 11)
    geps = 1.0 + 0.5 * rf
    gmu = np.ones_like(rf)
    gea = np.stack([0.8 * rf, 0.3 * rf ** 2], axis=1).ravel()
    c["geometry"] = [
        {"type": "two medium box", "center": [-1.5, 0.5, 0], "size": [5, 4, 3], "dimension": dim,
         "density dataset": "two medium box 0", "medium1": medium(12.0), "medium2": medium(1.0)},
        {"type": "general medium box", "center": [2.5, -1.0, 1.0], "size": [3, 4, 3], "dimension": gdim,
         "density dataset": "general medium box 1 density", "density function dataset": "general medium box 1 density function",
         "epsilon dataset": "general medium box 1 epsilon", "mu dataset": "general medium box 1 mu",
         "electric susceptibility amplitudes dataset": "general medium box 1 e sus amp",
         "magnetic susceptibility amplitudes dataset": "general medium box 1 m sus amp",
         "medium": medium(1.0, esus=[lorentz(0.1, 0.02, 1.0), drude(0.3, 0.05, 1.0)])},
    ]
    sdim = [4, 3, 1]
    samp = rng.uniform(0.2, 1.0, size=(sdim[2], sdim[1], sdim[0]))
    sph = rng.uniform(-np.pi, np.pi, size=(sdim[2], sdim[1], sdim[0]))
    c["sources"] = [{"type": "inhomogeneous source", "center": [0, 0, -3.5], "size": [3, 2, 0], "dimension": sdim,
                     "field component": "Ey", "amplitude dataset": "inhom source amplitude 0",
                     "phase dataset": "inhom source phase 0", "frequency": 0.1, "function": gauss1(0.1, 4.0, 8.0)}]
    c["fields output"] = [dft([-1.5, 0.5, 0], [5, 4, 3], comp, [0.1], k) for k, comp in enumerate(["Ex", "Ey", "Ez"])]
    c["fields output"].append(dft([2.5, -1.0, 1.0], [3, 4, 3], "Hz", [0.1, 0.12], 3))
    c["geometry info request"] = [{"field component": comp, "geometry index": 0,
                                   "output group": "geometry info request 0 %s" % comp} for comp in ["Ex", "Ey", "Ez"]]
    c["stop condition"] = {"type": "time", "time": 70}
    ds = {"two medium box 0": rho.ravel(), "general medium box 1 density": grho.ravel(),
          "general medium box 1 density function": rf, "general medium box 1 epsilon": geps,
          "general medium box 1 mu": gmu, "general medium box 1 e sus amp": gea,
          "general medium box 1 m sus amp": np.zeros(0), "inhom source amplitude 0": samp.ravel(),
          "inhom source phase 0": sph.ravel()}
    out["density_boxes"] = (c, ds)

    # 4. PMC symmetry in x, periodic y, CPML on z only; odd-size grid,
    #    resolution 2, Courant 0.4
    c = base([7.5, 6.0, 8.0], res=2.0, sc=0.4)
    c["symmetry"] = [{"direction": "x", "phase factor": 1}]
    c["periodic"] = [0, 1, 0]
    c["PML"] = [pml(1.5, 6.0, direction="z")]
    c["geometry"] = [{"type": "sphere", "center": [1.0, 0.5, 0.5], "radius": 1.3, "medium": medium(2.5)}]
    c["sources"] = [vsrc([0.5, 0.25, -2.0], [0, 0, 0], "Ez", 0.2), vsrc([2.25, -1.0, -2.5], [0, 0, 0], "Hy", 0.18, amp=0.5)]
    c["fields output"] = [dft([1.5, 0, 0.5], [3, 6, 5], "Ez", [0.15, 0.2], 0),
                          dft([1.5, 0, 0.5], [3, 6, 5], "Hx", [0.2], 1),
                          dft([1.5, 0, 0.5], [3, 6, 5], "Ey", [0.2], 2)]
    c["stop condition"] = {"type": "time", "time": 30}
    out["pmc_periodic_odd"] = (c, {})

    # 5. PEC symmetry in z, periodic x, CPML on y; magnetic media
    c = base([10, 12, 9])
    c["symmetry"] = [{"direction": "z", "phase factor": -1}]
    c["periodic"] = [1, 0, 0]
    c["PML"] = [pml(3, 4.0, direction="y", side="negative"), pml(2, 5.0, kmax=2.0, direction="y", side="positive")]
    c["geometry"] = [
        {"type": "box", "center": [0, 1, 2], "size": [4, 3, 2], "medium": medium(2.0, mu=1.5, mcond=0.02)},
        {"type": "sphere", "center": [-2.0, -1.0, 1.5], "radius": 1.8,
         "medium": medium(1.0, mu=1.2, msus=[lorentz(0.15, 0.02, 0.4)])},
    ]
    c["sources"] = [vsrc([0.2, -2.0, 1.3], [0, 0, 0], "Ex", 0.12), vsrc([1.0, 0.0, 2.7], [2, 0, 0], "Hz", 0.14)]
    c["fields output"] = [dft([0, 0, 2], [8, 8, 3], "Hx", [0.12, 0.14], 0),
                          dft([0, 0, 2], [8, 8, 3], "Ex", [0.12], 1),
                          dft([0, 0, 2], [8, 8, 3], "By", [0.12], 2)]
    c["stop condition"] = {"type": "time", "time": 45}
    out["pec_periodic_magnetic"] = (c, {})

    # 6. decay stop condition
    c = base([12, 12, 12])
    c["PML"] = [pml(3, 4.6)]
    c["sources"] = [vsrc([0, 0, 0.5], [0, 0, 0], "Ez", 0.15)]
    c["fields output"] = [dft([0, 0, 0], [4, 4, 4], "Ez", [0.15], 0)]
    c["stop condition"] = {"type": "decay", "position": [1.0, 0.5, 0.5], "field component": "Ez",
                           "time interval examined": 5.0, "decayed by": 1e-3}
    out["decay_stop"] = (c, {})

    # 7. DFT steady-state stop condition
    c = base([12, 12, 12])
    c["PML"] = [pml(3, 4.6)]
    c["geometry"] = [{"type": "box", "center": [0, 0, 1.5], "size": [6, 6, 2], "medium": medium(4.0)}]
    c["sources"] = [vsrc([0, 0, -2.0], [4, 4, 0], "Ey", 0.15)]
    c["fields output"] = [dft([0, 0, 3.0], [4, 4, 0], "Ey", [0.15, 0.13], 0)]
    c["stop condition"] = {"type": "dft", "center": [0, 0, 3.0], "size": [4, 4, 0], "field component": "Ey",
                           "time interval examined": 4.0, "variation": 1e-3, "frequency": 0.15}
    out["dft_stop"] = (c, {})
    return out


def run_case(binary, cfg, ds, workdir):
    ind = os.path.join(workdir, cfg["input file"] + ".d")
    os.makedirs(ind, exist_ok=True)
    for k, v in ds.items():
        np.save(os.path.join(ind, k + ".npy"), np.asarray(v, dtype=np.float64))
    with open(os.path.join(workdir, "config.json"), "w") as f:
        json.dump(cfg, f, indent=1)
    subprocess.run([binary], cwd=workdir, check=True, stdout=subprocess.DEVNULL)
    res = {}
    od = os.path.join(workdir, cfg["fields output file"] + ".d")
    for g in sorted(os.listdir(od)):
        for fn in sorted(os.listdir(os.path.join(od, g))):
            res[g + "/" + fn[:-4]] = np.load(os.path.join(od, g, fn))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FFIP_REFERENCE"), required="FFIP_REFERENCE" not in os.environ,
                    help="reference checkout (default: $FFIP_REFERENCE)")
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), "REF=" + a.ref])
    binary = os.path.join(ROOT, "oracle", "_ref", "run_sim_json")
    for name, (cfg, ds) in cases().items():
        wd = tempfile.mkdtemp(prefix="golden_")
        try:
            res = run_case(binary, cfg, ds, wd)
        finally:
            shutil.rmtree(wd, ignore_errors=True)
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump({"config": cfg, "datasets": {k: np.asarray(v).tolist() for k, v in ds.items()}}, f)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, len(res), "arrays")


if __name__ == "__main__":
    sys.exit(main())
