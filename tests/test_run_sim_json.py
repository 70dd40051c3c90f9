"""The run_sim_json driver (config.json + .npy input directory in, .npy
output groups out) against the in-process C ABI, on the emulation library
(CPU) and, marked gpu, on the CUDA library."""

import numpy as np
import pytest

from golden_cases import load

emu = pytest.importorskip("emu.build_emu")


def _compare(tmp_path, name, exe, lib):
    from ffip_gb300 import native, runfiles
    cfg, ds, _ = load(name)
    d = runfiles.write_inputs(str(tmp_path / name), cfg, ds)
    r = runfiles.run(d, exe=exe, timeout=600)
    assert r.returncode == 0, r.stderr
    got = runfiles.read_outputs(d, cfg)
    want = native.run_json(cfg, ds, lib=lib)
    assert set(got) == set(want)
    for g in want:
        for a in want[g]:
            assert got[g][a].shape == want[g][a].shape, (g, a)
            assert np.array_equal(got[g][a], want[g][a]), (g, a)


@pytest.mark.parametrize("name", ["density_boxes", "vacuum_pml"])
def test_driver_matches_in_process_run_emulated(tmp_path, name):
    from ffip_gb300 import native
    _compare(tmp_path, name, emu.build_cli(), native.load(emu.build()))


def test_driver_reports_errors(tmp_path):
    from ffip_gb300 import runfiles
    cfg, ds, _ = load("density_boxes")
    d = runfiles.write_inputs(str(tmp_path / "bad"), cfg, {})   # datasets missing
    r = runfiles.run(d, exe=emu.build_cli(), timeout=600)
    assert r.returncode == 1
    assert "dataset not provided" in r.stderr


@pytest.mark.gpu
def test_driver_matches_in_process_run_gpu(tmp_path):
    from ffip_gb300 import native, runfiles
    _compare(tmp_path, "density_boxes", runfiles.CLI, native.load())
