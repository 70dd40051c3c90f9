"""CPU check of the engine's host logic (set-up, array layout, CPML tables,
media slots, source splatting, DFT monitors, ghost planes, stop conditions,
output assembly): the engine is linked with a host emulation backend that
runs the same per-point update functions as the CUDA kernels
(tests/emu/host_backend.cpp), and its outputs are compared with the
reference's golden outputs."""
import copy

import numpy as np
import pytest

from golden_cases import CASES, flatten, load

emu = pytest.importorskip("emu.build_emu")


@pytest.fixture(scope="module")
def lib():
    from ffip_gb300 import native
    return native.load(emu.build())


def rel_errors(out, ref):
    errs = {}
    for k, r in ref.items():
        assert k in out, k
        assert out[k].shape == r.shape, k
        if k.endswith("/real") or k.endswith("/imag"):
            g = k.rsplit("/", 1)[0]
            scale = max(np.abs(ref[g + "/real"]).max(), np.abs(ref[g + "/imag"]).max())
            errs[k] = np.abs(out[k] - r).max() / scale
        else:
            assert np.array_equal(out[k], r), k
    return errs


@pytest.mark.parametrize("name", CASES)
def test_emulated_fp64_matches_reference(lib, name):
    from ffip_gb300 import native
    cfg, ds, ref = load(name)
    errs = rel_errors(flatten(native.run_json(cfg, ds, lib=lib)), ref)
    assert max(errs.values()) <= 1e-10, errs


@pytest.mark.parametrize("name", ["vacuum_pml", "dispersive", "density_boxes", "pec_periodic_magnetic"])
def test_emulated_fp32_within_1e_4(lib, name):
    from ffip_gb300 import native
    cfg, ds, ref = load(name)
    cfg = copy.deepcopy(cfg)
    cfg["precision"] = "fp32"
    errs = rel_errors(flatten(native.run_json(cfg, ds, lib=lib)), ref)
    assert max(errs.values()) <= 1e-4, errs


def test_set_density_equals_fresh_run(lib):
    from ffip_gb300 import native
    cfg, ds, _ = load("density_boxes")
    rho2 = np.random.default_rng(5).uniform(0, 1, size=ds["two medium box 0"].shape)
    ds2 = dict(ds)
    ds2["two medium box 0"] = rho2
    fresh = flatten(native.run_json(cfg, ds2, lib=lib))
    with native.NativeSim(cfg, ds, lib=lib) as s:
        s.run(cfg["stop condition"])
        s.set_density("two medium box 0", rho2)
        assert s.stats()["time_step"] == 0
        s.run(cfg["stop condition"])
        again = flatten(s.outputs())
    for k in fresh:
        assert np.array_equal(fresh[k], again[k]), k


def test_set_source_data_equals_fresh_run(lib):
    from ffip_gb300 import native
    cfg, ds, _ = load("density_boxes")
    rng = np.random.default_rng(9)
    amp = rng.uniform(0.5, 2.0, size=ds["inhom source amplitude 0"].shape)
    phase = rng.uniform(-np.pi, np.pi, size=ds["inhom source phase 0"].shape)
    ds2 = dict(ds)
    ds2["inhom source amplitude 0"] = amp
    ds2["inhom source phase 0"] = phase
    fresh = flatten(native.run_json(cfg, ds2, lib=lib))
    with native.NativeSim(cfg, ds, lib=lib) as s:
        s.run(cfg["stop condition"])
        s.set_source_data({"inhom source amplitude 0": amp, "inhom source phase 0": phase})
        assert s.stats()["time_step"] == 0
        s.run(cfg["stop condition"])
        again = flatten(s.outputs())
        with pytest.raises(native.FfipError, match="no inhomogeneous source"):
            s.set_source_data({"two medium box 0": amp})
        with pytest.raises(native.FfipError, match="values"):
            s.set_source_data({"inhom source amplitude 0": amp[:-1]})
    for k in fresh:
        assert np.array_equal(fresh[k], again[k]), k


def test_large_design_workload_builds_and_steps(lib):
    """The large design workload's configuration (Drude backplane, Lorentz /
    vacuum density box, three DFT planes at many frequencies), scaled down,
    builds and steps on the emulated engine with slots from both media."""
    from ffip_gb300 import native, workloads
    cfg, ds = workloads.large_design(n=48, nz=40, pml=6, design=(24, 6), nfreq=4, steps=10, precision="fp32")
    with native.NativeSim(cfg, ds, lib=lib) as s:
        s.run()
        out = s.outputs()
        st = s.stats()
    assert st["time_step"] == 10 and st["yee_cells"] == 48 * 48 * 40
    groups = [g for g in out if g.startswith("volume fields dft")]
    assert len(groups) == 3
    for g in groups:
        assert out[g]["real"].shape[0] == 4


def test_step_timed_pass_steps_like_step(lib):
    """ffip_step_timed_pass through the C ABI: the same steps as ffip_step
    (same outputs, same time step), and a pass time of 0 where the backend
    does not time fused passes (the host emulation runs separate passes)."""
    from ffip_gb300 import native
    cfg, ds, _ = load("vacuum_pml")
    steps = 37
    outs = []
    for timed in (False, True):
        s = native.NativeSim(cfg, ds, lib=lib)
        try:
            if timed:
                ms, pms = s.step_timed_pass(steps)
                assert ms >= 0 and pms == 0
            else:
                s.step(steps)
            st = s.stats()
            assert st["time_step"] == steps
            assert 0 < st["pass_bytes_per_step"] <= st["bytes_per_step"]
            outs.append(flatten(s.outputs()))
        finally:
            s.close()
    for k in outs[0]:
        assert np.array_equal(outs[0][k], outs[1][k]), k
    with pytest.raises(native.FfipError):
        s = native.NativeSim(cfg, ds, lib=lib)
        try:
            s.step_timed_pass(-1)
        finally:
            s.close()


@pytest.mark.parametrize("precision,steps", [("fp32", 200), ("fp64", 1300)])
def test_divergence_check_stops_the_unstable_debye_run(lib, precision, steps):
    """The reference's Debye pole is unconditionally unstable: run long, the
    fields overflow, and a check every 100 steps stops the run with
    FFIP_ERR_DIVERGED at the first check that sees non-finite values; with
    the check off the run goes on and its outputs carry them."""
    from ffip_gb300 import native
    cfg, ds, _ = load("debye_short")
    cfg = copy.deepcopy(cfg)
    cfg["precision"] = precision
    cfg["divergence check interval"] = 100
    with native.NativeSim(cfg, ds, lib=lib) as s:
        with pytest.raises(native.FfipError, match=r"error -5: the simulation diverged.*time step %d " % steps):
            s.step(3000)
        assert s.stats()["time_step"] == steps
    cfg["divergence check interval"] = 0
    with native.NativeSim(cfg, ds, lib=lib) as s:
        s.step(steps + 100)
        out = flatten(s.outputs())
        assert not all(np.isfinite(v).all() for k, v in out.items() if k.endswith("/real"))


def test_divergence_check_interval_is_validated(lib):
    from ffip_gb300 import native
    cfg, ds, _ = load("vacuum_pml")
    for bad in (-1, 2.5):
        c = copy.deepcopy(cfg)
        c["divergence check interval"] = bad
        with pytest.raises(native.FfipError, match="divergence check interval"):
            native.NativeSim(c, ds, lib=lib)
    c = copy.deepcopy(cfg)
    c["fused wait timeout"] = 0
    with pytest.raises(native.FfipError, match="fused wait timeout"):
        native.NativeSim(c, ds, lib=lib)


@pytest.mark.parametrize("seed", range(8))
def test_emulated_random_boundaries_match_oracle(lib, seed):
    """Seeded PEC / PMC / periodic / CPML faces on odd and even grids
    (tests/test_gpu_parity.py random_boundary_config): the host logic of the
    ghost faces against the oracle, whole-grid monitors of all six
    components, 1e-10."""
    from ffip_gb300 import native
    from oracle import port
    from test_gpu_parity import random_boundary_config
    cfg = random_boundary_config(seed)
    out = flatten(native.run_json(cfg, {}, lib=lib))
    ref = flatten(port.run_json(cfg, {}, threads=4))
    errs = rel_errors(out, ref)
    assert all(np.abs(out[k]).max() > 0 for k in out if k.endswith("/real"))
    assert max(errs.values()) <= 1e-10, errs


def partition_check(lib, cfg):
    """The host half of the fused pass's split of a step (fused_plan.hpp) on
    a config's plan: every valid point owned by the pass or in exactly one
    face box, and no E point of the pass reading an H ghost unless its face
    is mirrored into the halo of the first tiles (tests/emu/host_backend.cpp)."""
    import ctypes
    import json
    fn = lib.ffip_emu_fused_partition_check
    fn.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint64]
    fn.restype = ctypes.c_int
    msg = ctypes.create_string_buffer(512)
    rc = fn(json.dumps(cfg).encode(), msg, 512)
    return rc, msg.value.decode()


@pytest.mark.parametrize("seed", range(24))
def test_fused_partition_on_random_boundaries(lib, seed):
    from test_gpu_parity import random_boundary_config
    rc, msg = partition_check(lib, random_boundary_config(seed))
    assert rc == 0, msg


def test_fused_partition_on_golden_cases_and_workloads(lib):
    """Golden cases (PMC / PEC symmetry with periodic faces, odd grids) and
    the spheres workload at 33 and 40 cells with every kind of face."""
    from ffip_gb300 import workloads
    cfgs = [cfg for cfg, ds, _ in (load(n) for n in CASES) if not ds]  # (the hook takes no datasets)
    for n in (33, 40):
        cfg = workloads.dispersive_spheres(n, steps=10)
        cfgs.append(cfg)
        for sym, per in (([{"direction": "x", "phase factor": 1}], [0, 1, 0]), ([{"direction": "y", "phase factor": -1}], [1, 0, 1]),
                         ([{"direction": "x", "phase factor": -1}, {"direction": "y", "phase factor": 1}], [1, 1, 1])):
            c = copy.deepcopy(cfg)
            c["symmetry"], c["periodic"] = sym, per
            cfgs.append(c)
    mirrored = 0
    for cfg in cfgs:
        rc, msg = partition_check(lib, cfg)
        assert rc == 0, msg
        mirrored += "mirror 0 0" not in msg
    assert mirrored >= 6  # the symmetry faces along x / y are mirrored, not deferred


def jobs_check(lib, cfg, tx, kch):
    """The fused pass's CTA job lists (fused_plan.hpp fused_jobs) on a
    config's plan: every unit / tile / plane in exactly one job, no
    CPML-free job meeting CPML (tests/emu/host_backend.cpp)."""
    import ctypes
    import json
    fn = lib.ffip_emu_fused_jobs_check
    fn.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_uint64]
    fn.restype = ctypes.c_int
    msg = ctypes.create_string_buffer(512)
    rc = fn(json.dumps(cfg).encode(), tx, kch, msg, 512)
    return rc, msg.value.decode()


@pytest.mark.parametrize("tx", [32, 64])
@pytest.mark.parametrize("kch", [4, 12, 16])
def test_fused_jobs_cover_the_grid(lib, tx, kch):
    """The spheres workload at 64, 128 and 256 cells (CPML on every face,
    spheres with slots, the DFT volume), the plain vacuum box and seeded
    random boundary configurations; the interior instance's tile is 64
    columns wide in fp32, 32 in fp64."""
    from ffip_gb300 import workloads
    from test_gpu_parity import random_boundary_config
    cfgs = [workloads.dispersive_spheres(n, steps=10) for n in (64, 128, 256)] + [workloads.vacuum_point(64)]
    cfgs += [random_boundary_config(s) for s in range(8)]
    interior = 0
    for cfg in cfgs:
        rc, msg = jobs_check(lib, cfg, tx, kch)
        assert rc == 0, msg
        interior += int(msg.split(" CPML jobs, ")[1].split()[0])
    assert interior > 0  # the larger grids put jobs on the instance without CPML code
