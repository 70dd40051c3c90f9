"""GPU parity: the CUDA path, called through the C ABI (include/ffip_gb300.h),
against the reference's golden outputs and against the oracle on seeded
random configurations.

Tolerances (relative to the largest |DFT| of the monitor group):
  fp64 state:  1e-10  (the drop-in bar)
  fp32 state:  1e-4   (fp32 fields, fp64 DFT sums)
"""
import copy

import numpy as np
import pytest

from golden_cases import CASES, flatten, load

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
FP32_TOL = 1e-4


def rel_err(out, ref):
    worst = 0.0
    for k, r in ref.items():
        assert k in out, k
        assert out[k].shape == r.shape, (k, out[k].shape, r.shape)
        if k.endswith("/real") or k.endswith("/imag"):
            g = k.rsplit("/", 1)[0]
            scale = max(np.abs(ref[g + "/real"]).max(), np.abs(ref[g + "/imag"]).max())
            worst = max(worst, np.abs(out[k] - r).max() / scale)
        else:
            assert np.array_equal(out[k], r), k
    return worst


def gpu_run(cfg, ds=None, **over):
    from ffip_gb300 import native
    cfg = copy.deepcopy(cfg)
    cfg.update(over)
    return flatten(native.run_json(cfg, ds or {}))


@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference(name):
    cfg, ds, ref = load(name)
    assert rel_err(gpu_run(cfg, ds, precision="fp64"), ref) <= FP64_TOL


@pytest.mark.parametrize("name", CASES)
def test_fp32_within_tolerance(name):
    cfg, ds, ref = load(name)
    assert rel_err(gpu_run(cfg, ds, precision="fp32"), ref) <= FP32_TOL


FUSED_ELIGIBLE = ["vacuum_pml", "dispersive", "debye_short", "density_boxes", "decay_stop", "dft_stop", "pmc_periodic_odd",
                  "pec_periodic_magnetic"]


@pytest.mark.parametrize("name", FUSED_ELIGIBLE)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_pass_is_bitwise_equal_to_separate_passes(name, precision):
    """The fused H+E kernel runs the same per-point arithmetic in the same
    order as the separate H and E kernels, so results must agree exactly."""
    from ffip_gb300 import native
    cfg, ds, _ = load(name)
    cfg = copy.deepcopy(cfg)
    cfg["precision"] = precision
    outs = {}
    for eng in ("unfused", "fused"):
        c = copy.deepcopy(cfg)
        c["engine"] = eng
        with native.NativeSim(c, ds) as s:
            assert s.stats()["fused"] == (1 if eng == "fused" else 0)
            s.run(c["stop condition"])
            outs[eng] = flatten(s.outputs())
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k


def test_auto_engine_picks_the_fused_pass():
    """Every boundary kind and medium, magnetic poles included."""
    from ffip_gb300 import native
    for name in ("vacuum_pml", "pmc_periodic_odd", "pec_periodic_magnetic"):
        cfg, ds, _ = load(name)
        with native.NativeSim(cfg, ds) as s:
            assert s.stats()["fused"] == 1, name
    cfg, ds, _ = load("vacuum_pml")
    cfg = copy.deepcopy(cfg)
    cfg["engine"] = "unfused"
    with native.NativeSim(cfg, ds) as s:
        assert s.stats()["fused"] == 0


def _without_magnetic_poles(cfg):
    """Magnetic susceptibilities and magnetic conductivity (a pole with
    a0 = b1 = 1, as in the reference's json2medium) removed; mu kept."""
    cfg = copy.deepcopy(cfg)
    for g in cfg.get("geometry", []):
        for key in ("medium", "medium1", "medium2"):
            if key in g:
                g[key]["magnetic susceptibility"] = []
                g[key]["magnetic conductivity"] = 0.0
    return cfg


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_pec_periodic_magnetic_media_match_separate_passes(precision):
    """PEC symmetry along z (both faces, with periodic z), periodic x, CPML of
    different thickness on the two y faces, mu != 1 and an Hz source, with H
    slots that hold no pole (the golden case's magnetic pole and magnetic
    conductivity dropped; the case itself runs in FUSED_ELIGIBLE)."""
    from ffip_gb300 import native
    cfg, ds, _ = load("pec_periodic_magnetic")
    cfg = _without_magnetic_poles(cfg)
    cfg["precision"] = precision
    cfg["periodic"] = [1, 0, 1]
    outs = {}
    for eng in ("unfused", "fused"):
        c = copy.deepcopy(cfg)
        c["engine"] = eng
        with native.NativeSim(c, ds) as s:
            assert s.stats()["fused"] == (1 if eng == "fused" else 0)
            s.run(c["stop condition"])
            outs[eng] = flatten(s.outputs())
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k
    assert max(np.abs(v).max() for k, v in outs["fused"].items() if k.endswith("/real")) > 0


def _boundary_variant(kind, precision):
    """The 96^3 dispersive-spheres workload (120 steps) with PEC / PMC /
    periodic faces: CPML only along the axes without them, an Hz source, and
    whole-grid DFT monitors of Ey and Hz so that the E and H layers next to
    every face are compared."""
    from ffip_gb300 import workloads
    cfg = workloads.dispersive_spheres(96, steps=120, precision=precision)
    pml = cfg["PML"][0]
    if kind == "pmc_x_periodic_y":
        cfg["symmetry"] = [{"direction": "x", "phase factor": 1}]
        cfg["periodic"] = [0, 1, 0]
        axes = ["z"]
    elif kind == "odd_periodic_xz_pec_y":
        # odd cell counts: the low faces start at odd doubled coordinates
        cfg["size"] = [93.0, 90.0, 87.0]
        cfg["symmetry"] = [{"direction": "y", "phase factor": -1}]
        cfg["periodic"] = [1, 0, 1]
        axes = []
    elif kind == "magnetic_pmc_x_periodic_y":
        # magnetic Lorentz poles and magnetic conductivity in every third
        # sphere, and a magnetic sphere around the Hz source (its current
        # waits at a slot with poles until the H update)
        cfg["symmetry"] = [{"direction": "x", "phase factor": 1}]
        cfg["periodic"] = [0, 1, 0]
        axes = ["z"]
        msus = [{"type": "Lorentz", "frequency": 0.11, "gamma": 0.02, "amplitude": 0.6}]
        for i, g in enumerate(cfg["geometry"]):
            if i % 3 == 0:
                g["medium"] = dict(g["medium"], mu=1.4, **{"magnetic susceptibility": msus, "magnetic conductivity": 0.01})
        cfg["geometry"].insert(0, {"type": "sphere", "center": [5.0, -7.0, 3.0], "radius": 4.0,
                                   "medium": dict(cfg["geometry"][0]["medium"], **{"magnetic susceptibility": msus})})
        cfg["fields output"].append({"type": "volume fields dft", "center": [0.0, 0.0, 0.0], "size": list(cfg["size"]),
                                     "frequency": [0.1], "field component": "By", "output group": "whole grid By"})
    else:  # pec_z_both_faces_pml_xy
        cfg["symmetry"] = [{"direction": "z", "phase factor": -1}]
        cfg["periodic"] = [0, 0, 1]
        axes = ["x", "y"]
    cfg["PML"] = [dict(pml, direction=a) for a in axes]
    cfg["sources"].append({"type": "volume source", "center": [5.0, -7.0, 3.0], "size": [0.0, 0.0, 0.0], "amplitude": 1.0,
                           "field component": "Hz",
                           "function": {"type": "Gaussian1", "frequency": 0.12, "cutoff": 4.0, "start time": 0.0}})
    for comp in ("Ey", "Hz"):
        cfg["fields output"].append({"type": "volume fields dft", "center": [0.0, 0.0, 0.0], "size": list(cfg["size"]),
                                     "frequency": [0.1], "field component": comp, "output group": "whole grid " + comp})
    return cfg


@pytest.mark.parametrize("kind", ["pmc_x_periodic_y", "odd_periodic_xz_pec_y", "pec_z_both_faces_pml_xy",
                                  "magnetic_pmc_x_periodic_y"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_boundary_faces_large_grid_match_separate_passes(kind, precision):
    """Several x units, y tiles and z chunks with ghost faces of each kind on
    both lo parities: the fused pass (with the E layers next to H ghost
    planes left to the face kernel) equals the separate passes bit for bit."""
    from ffip_gb300 import native
    outs = {}
    for eng in ("unfused", "fused"):
        cfg = _boundary_variant(kind, precision)
        cfg["engine"] = eng
        with native.NativeSim(cfg, {}) as s:
            assert s.stats()["fused"] == (1 if eng == "fused" else 0)
            s.run(cfg["stop condition"])
            outs[eng] = flatten(s.outputs())
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k
    assert np.abs(outs["fused"]["whole grid Hz/real"]).max() > 0


def test_fused_large_grid_matches_separate_passes():
    """Several z chunks and x/y tiles, CPML, spheres and the sheet source."""
    from ffip_gb300 import native, workloads
    outs = {}
    for eng in ("unfused", "fused"):
        cfg = workloads.dispersive_spheres(96, steps=120, precision="fp32", engine=eng)
        outs[eng] = flatten(native.run_json(cfg))
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k


def test_repeat_runs_are_bitwise_identical():
    cfg, ds, _ = load("dispersive")
    a = gpu_run(cfg, ds)
    b = gpu_run(cfg, ds)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def random_config(seed, n=20, steps=150):
    """Seeded random media/sources/monitors in the reference's schema."""
    rng = np.random.default_rng(seed)
    med = lambda eps, esus=(): {"epsilon": eps, "mu": 1.0, "electric conductivity": 0.0, "magnetic conductivity": 0.0,
                                "electric susceptibility": list(esus), "magnetic susceptibility": []}
    geoms = []
    for g in range(6):
        kind = rng.integers(0, 3)
        esus = []
        if kind == 1:
            esus = [{"type": "Lorentz", "frequency": float(rng.uniform(0.05, 0.2)), "gamma": float(rng.uniform(0.001, 0.02)),
                     "amplitude": float(rng.uniform(0.5, 3))}]
        elif kind == 2:
            esus = [{"type": "Drude", "frequency": float(rng.uniform(0.05, 0.2)), "gamma": float(rng.uniform(0.005, 0.05)),
                     "amplitude": 1.0}]
        geoms.append({"type": "sphere", "center": [float(v) for v in rng.uniform(-5, 5, 3)], "radius": float(rng.uniform(1, 4)),
                      "medium": med(float(rng.uniform(1, 4)), esus)})
    comps = ["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"]
    return {
        "courant number": 0.5, "resolution": 1.0, "size": [n, n, n], "input file": "x", "fields output file": "y",
        "default material": med(1.0),
        "PML": [{"thickness": 4.0, "k max": 1.0, "sigma max": 3.45, "order": 3}],
        "geometry": geoms,
        "sources": [{"type": "volume source", "center": [float(v) for v in rng.uniform(-3, 3, 3)], "size": [0, 0, 0],
                     "amplitude": 1.0, "field component": comps[int(rng.integers(0, 6))],
                     "function": {"type": "Gaussian1", "frequency": 0.1, "cutoff": 4.0, "start time": 0.0}}],
        "fields output": [{"type": "volume fields dft", "center": [0, 0, 0], "size": [8, 8, 8], "frequency": [0.08, 0.1, 0.12],
                           "field component": c, "output group": "volume fields dft %d" % i} for i, c in enumerate(comps)],
        "stop condition": {"type": "time", "time": steps * 0.5},
    }


def random_boundary_config(seed, steps=120):
    """random_config with seeded boundaries: per axis PEC or PMC symmetry,
    periodic, both, or CPML (on one or both faces), odd and even cell counts,
    resolution 1 or 2."""
    rng = np.random.default_rng(1000 + seed)
    cfg = random_config(seed, steps=steps)
    cfg["resolution"] = float(rng.choice([1.0, 2.0]))
    cfg["size"] = [float(rng.integers(9, 14) + rng.choice([0.0, 0.5])) for _ in range(3)]
    sym, per, pml = [], [0, 0, 0], []
    for a, d in enumerate("xyz"):
        kind = rng.choice(["pec", "pmc", "periodic", "pec_periodic", "cpml", "cpml_one"])
        if kind in ("pec", "pmc", "pec_periodic"):
            sym.append({"direction": d, "phase factor": -1 if kind != "pmc" else 1})
        if kind in ("periodic", "pec_periodic"):
            per[a] = 1
        if kind == "cpml":
            pml.append({"thickness": 2.0, "k max": 1.0, "sigma max": 3.45, "order": 3, "direction": d})
        if kind == "cpml_one":
            pml.append({"thickness": 2.0, "k max": 1.0, "sigma max": 3.45, "order": 3, "direction": d,
                        "side": str(rng.choice(["negative", "positive"]))})
    cfg["symmetry"], cfg["periodic"], cfg["PML"] = sym, per, pml
    for g in cfg["geometry"]:
        g["center"] = [float(v) for v in rng.uniform(-3, 3, 3)]
        g["radius"] = float(rng.uniform(1, 3))
    # a symmetry face puts the grid on the positive side only (lo = 0)
    symmetric = {d["direction"] for d in sym}
    cfg["sources"][0]["center"] = [float(rng.uniform(0.6, 2.0) if d in symmetric else rng.uniform(-2, 2)) for d in "xyz"]
    cfg["fields output"] = [dict(m, size=[float(v) for v in cfg["size"]]) for m in cfg["fields output"]]
    return cfg


@pytest.mark.parametrize("seed", range(8))
def test_fused_random_boundaries_match_separate_passes_and_oracle(seed):
    """Random PEC / PMC / periodic / CPML faces: the fused pass equals the
    separate passes bit for bit and the oracle to 1e-10, with whole-grid
    monitors of all six components."""
    from ffip_gb300 import native
    from oracle import port
    cfg = random_boundary_config(seed)
    outs = {}
    for eng in ("unfused", "fused"):
        c = copy.deepcopy(cfg)
        c["engine"] = eng
        c["precision"] = "fp64"
        with native.NativeSim(c) as s:
            assert s.stats()["fused"] == (1 if eng == "fused" else 0)
            s.run(c["stop condition"])
            outs[eng] = flatten(s.outputs())
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k
    assert all(np.abs(v).max() > 0 for k, v in outs["fused"].items() if k.endswith("/real"))
    ref = flatten(port.run_json(cfg, {}, threads=4))
    assert rel_err(outs["fused"], ref) <= FP64_TOL


@pytest.mark.parametrize("thin_axis", [0, 1, 2])
@pytest.mark.parametrize("thin", [0.5, 1.0, 2.0])
@pytest.mark.parametrize("resolution", [1.0, 2.0])
def test_fused_thin_periodic_grids_match_separate_passes_and_oracle(thin_axis, thin, resolution):
    """Two-dimensional-like grids: one or two cells along a periodic axis
    (fewer planes than a z chunk or tile), CPML along the other two; fused
    equals separate passes bit for bit and the oracle to 1e-10 (monitor
    groups that are zero by symmetry must be zero)."""
    from ffip_gb300 import native
    from oracle import port
    cfg = random_config(3, n=14, steps=80)
    size = [14.0, 12.0, 10.0]
    size[thin_axis] = thin
    cfg["size"], cfg["resolution"] = size, resolution
    cfg["periodic"] = [1 if a == thin_axis else 0 for a in range(3)]
    cfg["PML"] = [{"thickness": 2.0, "k max": 1.0, "sigma max": 3.45, "order": 3, "direction": d}
                  for a, d in enumerate("xyz") if a != thin_axis]
    cfg["sources"][0]["center"] = [0.3, -0.4, 0.2]
    cfg["fields output"] = [dict(m, size=list(size)) for m in cfg["fields output"]]
    outs = {}
    for eng in ("unfused", "fused"):
        c = copy.deepcopy(cfg)
        c["engine"] = eng
        with native.NativeSim(c) as s:
            assert s.stats()["fused"] == (1 if eng == "fused" else 0)
            s.run(c["stop condition"])
            outs[eng] = flatten(s.outputs())
    for k in outs["unfused"]:
        assert np.array_equal(outs["unfused"][k], outs["fused"][k]), k
    ref = flatten(port.run_json(cfg, {}, threads=4))
    for k, r in ref.items():
        g = k.rsplit("/", 1)[0]
        if (k.endswith("/real") or k.endswith("/imag")) and max(np.abs(ref[g + "/real"]).max(), np.abs(ref[g + "/imag"]).max()) == 0:
            assert not np.abs(outs["fused"][k]).any(), k
            del outs["fused"][k]
    ref = {k: v for k, v in ref.items() if k in outs["fused"]}
    assert rel_err(outs["fused"], ref) <= FP64_TOL


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fp64_matches_oracle_on_random_configs(seed):
    from oracle import port
    cfg = random_config(seed)
    ref = flatten(port.run_json(cfg, {}, threads=4))
    assert rel_err(gpu_run(cfg, precision="fp64"), ref) <= FP64_TOL


def test_workload_downscaled_fp64_matches_oracle():
    """The benchmark workload (dispersive spheres) at 64^3, 300 steps."""
    from ffip_gb300 import workloads
    from oracle import port
    cfg = workloads.dispersive_spheres(64, steps=300, precision="fp64")
    ref = flatten(port.run_json(cfg, {}, threads=8))
    assert rel_err(gpu_run(cfg), ref) <= FP64_TOL
    cfg32 = workloads.dispersive_spheres(64, steps=300, precision="fp32")
    assert rel_err(gpu_run(cfg32), ref) <= FP32_TOL


def test_empty_and_outside_monitors():
    """A monitor outside the grid gives zeros of the closure shape, like the
    reference's unwritten HDF5 hyperslab."""
    cfg, ds, _ = load("vacuum_pml")
    cfg = copy.deepcopy(cfg)
    cfg["fields output"].append({"type": "volume fields dft", "center": [30, 30, 30], "size": [2, 2, 2], "frequency": [0.1],
                                 "field component": "Ey", "output group": "outside"})
    out = gpu_run(cfg, ds)
    from oracle import port
    ref = flatten(port.run_json(cfg, ds))
    assert out["outside/real"].shape == ref["outside/real"].shape
    assert not out["outside/real"].any()
    assert np.array_equal(out["outside/x"], ref["outside/x"])


def test_set_density_matches_fresh_create():
    from ffip_gb300 import native
    cfg, ds, _ = load("density_boxes")
    rho2 = np.random.default_rng(9).uniform(0, 1, size=ds["two medium box 0"].shape)
    ds2 = dict(ds)
    ds2["two medium box 0"] = rho2
    fresh = flatten(native.run_json(cfg, ds2))
    with native.NativeSim(cfg, ds) as s:
        s.run(cfg["stop condition"])
        s.set_density("two medium box 0", rho2)
        s.run(cfg["stop condition"])
        again = flatten(s.outputs())
    for k in fresh:
        assert np.array_equal(fresh[k], again[k]), k


def test_bad_device_index_is_an_error():
    from ffip_gb300 import native
    cfg, ds, _ = load("vacuum_pml")
    cfg = copy.deepcopy(cfg)
    cfg["device"] = 999
    with pytest.raises(native.FfipError):
        native.NativeSim(cfg, ds)


def test_fused_asymmetric_cpml_and_odd_sizes_match_separate_passes():
    """CPML on some faces only, odd sizes, a monitor and a sphere: the split
    of the fused pass into CPML / interior jobs and the face layers cover the
    grid exactly once."""
    from ffip_gb300 import native
    cfg = random_config(7, n=20, steps=80)
    cfg["size"] = [67.0, 41.0, 59.0]
    cfg["PML"] = [{"thickness": 6.0, "direction": "z", "side": "negative", "k max": 1.0, "sigma max": 3.0, "order": 3},
                  {"thickness": 9.0, "direction": "x", "k max": 2.0, "sigma max": 2.0, "order": 2}]
    outs = {}
    for eng in ("unfused", "fused"):
        for prec in ("fp64", "fp32"):
            c = dict(cfg)
            c["engine"] = eng
            c["precision"] = prec
            with native.NativeSim(c) as s:
                assert s.stats()["fused"] == (1 if eng == "fused" else 0)
                s.run(c["stop condition"])
                outs[eng, prec] = flatten(s.outputs())
    for prec in ("fp64", "fp32"):
        for k in outs["unfused", prec]:
            assert np.array_equal(outs["unfused", prec][k], outs["fused", prec][k]), (prec, k)


def test_fused_cpml_kappa_and_resolution_match_separate_passes():
    """CPML with k max > 1, one layer with sigma max = 0 (c = 0 but 1/k != 1:
    the reference leaves those points to the plain curl update), resolution 2
    (1/dx != 1): tile planes with CPML along one axis take the per-axis copy
    of the lean path in fp64; fused and separate passes give the same bits."""
    from ffip_gb300 import native
    cfg = random_config(11, n=20, steps=60)
    cfg["resolution"] = 2.0
    cfg["size"] = [21.0, 18.0, 22.0]
    cfg["PML"] = [{"thickness": 2.0, "direction": "y", "k max": 2.0, "sigma max": 0.0, "order": 3},
                  {"thickness": 3.0, "direction": "x", "side": "positive", "k max": 3.0, "sigma max": 2.5, "order": 2},
                  {"thickness": 2.5, "direction": "z", "k max": 1.0, "sigma max": 3.0, "order": 3}]
    outs = {}
    for eng in ("unfused", "fused"):
        for prec in ("fp64", "fp32"):
            c = dict(cfg)
            c["engine"] = eng
            c["precision"] = prec
            with native.NativeSim(c) as s:
                assert s.stats()["fused"] == (1 if eng == "fused" else 0)
                s.run(c["stop condition"])
                outs[eng, prec] = flatten(s.outputs())
    for prec in ("fp64", "fp32"):
        for k in outs["unfused", prec]:
            assert np.array_equal(outs["unfused", prec][k], outs["fused", prec][k]), (prec, k)
        assert max(np.abs(v).max() for k, v in outs["fused", prec].items() if k.endswith("/real")) > 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("case,steps", [("dispersive", None), ("vacuum_pml", 2100)])
def test_pass_timing_leaves_results_unchanged(precision, case, steps):
    """ffip_step_timed_pass brackets every fused pass with timing events (a
    pool of 1024 pairs, folded into a running sum when full: 2100 steps fold
    twice): the DFT sums equal those of plain ffip_step, and the summed pass
    time lies inside the steps' device time."""
    from ffip_gb300 import native
    cfg, ds, _ = load(case)
    cfg = copy.deepcopy(cfg)
    cfg["precision"] = precision
    if steps is None:
        steps = int(round(cfg["stop condition"]["time"] / (cfg["courant number"] / cfg["resolution"])))
    outs = []
    for timed in (False, True):
        s = native.NativeSim(cfg, ds)
        try:
            assert s.stats()["fused"] == 1
            if timed:
                ms, pms = s.step_timed_pass(steps)
                assert 0 < pms <= ms
                assert 0 < s.stats()["pass_bytes_per_step"] < s.stats()["bytes_per_step"]
            else:
                s.step(steps)
            outs.append(flatten(s.outputs()))
        finally:
            s.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k
