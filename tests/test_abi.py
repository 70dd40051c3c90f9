"""The C ABI library builds for sm_103a, loads, and exports every function
that include/ffip_gb300.h declares; argument and config errors come back as
error codes with messages (no GPU needed: they fail before any CUDA call)."""
import ctypes
import json
import os
import re


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(name="ffip_gb300.h"):
    txt = open(os.path.join(ROOT, "include", name)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ffip_[a-z_]+)\s*\(", txt)))


def test_header_declares_expected_entry_points():
    fns = header_functions()
    for f in ["ffip_create", "ffip_step", "ffip_run", "ffip_output_count", "ffip_output_array", "ffip_destroy",
              "ffip_last_error", "ffip_transpose", "ffip_sensitivity", "ffip_set_density"]:
        assert f in fns


def test_library_exports_every_declared_symbol():
    from ffip_gb300 import native
    lib = native.load()
    for f in header_functions():
        assert hasattr(lib, f), f
    assert sorted(native.EXPORTS) == header_functions()
    for f in header_functions("ffip_gb300_surrogate.h"):
        assert hasattr(lib, f), f


def test_build_targets_sm_103a_only():
    from ffip_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def _create(cfg_text):
    from ffip_gb300 import native
    lib = native.load()
    h = ctypes.c_void_p()
    rc = lib.ffip_create(cfg_text.encode(), None, 0, ctypes.byref(h))
    return rc, lib.ffip_last_error().decode()


def test_bad_json_is_an_error():
    rc, msg = _create("{not json")
    assert rc == -1 and "json" in msg


def test_missing_key_is_an_error():
    rc, msg = _create(json.dumps({"size": [4, 4, 4]}))
    assert rc == -1 and "resolution" in msg


def test_unstable_courant_is_rejected():
    rc, msg = _create(json.dumps({"size": [4, 4, 4], "resolution": 1, "courant number": 0.7}))
    assert rc == -1 and "courant" in msg


def test_unknown_susceptibility_is_an_error():
    cfg = {"size": [4, 4, 4], "resolution": 1,
           "default material": {"epsilon": 1, "mu": 1, "electric susceptibility": [{"type": "Cauchy", "amplitude": 1}]}}
    rc, msg = _create(json.dumps(cfg))
    assert rc == -1 and "susceptibility" in msg


def test_missing_dataset_is_an_error():
    cfg = {"size": [4, 4, 4], "resolution": 1,
           "geometry": [{"type": "two medium box", "center": [0, 0, 0], "size": [2, 2, 2], "dimension": [2, 2, 2],
                         "density dataset": "rho", "medium1": {"epsilon": 2, "mu": 1}, "medium2": {"epsilon": 1, "mu": 1}}]}
    rc, msg = _create(json.dumps(cfg))
    assert rc == -1 and "rho" in msg


def test_null_handle_calls_fail_cleanly():
    from ffip_gb300 import native
    lib = native.load()
    assert lib.ffip_step(None, 1) == -1
    assert lib.ffip_destroy(None) == 0
