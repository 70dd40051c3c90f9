"""Pins the oracle (oracle/port.py + oracle/step.c) to the reference itself:
every output array the reference's own code wrote for each golden case
(tests/golden/make_golden.py) must be reproduced bit for bit."""
import numpy as np
import pytest

from golden_cases import CASES, flatten, load
from oracle import port


@pytest.mark.parametrize("name", CASES)
def test_port_matches_reference_bitwise(name):
    cfg, ds, ref = load(name)
    out = flatten(port.run_json(cfg, ds))
    assert sorted(out) == sorted(ref)
    for k, r in ref.items():
        assert out[k].shape == r.shape, k
        assert np.array_equal(out[k], r), (k, np.abs(out[k] - r).max(), np.abs(r).max())


@pytest.mark.parametrize("name", ["dispersive", "pmc_periodic_odd"])
def test_port_thread_count_does_not_change_results(name):
    cfg, ds, _ = load(name)
    a = flatten(port.run_json(cfg, ds, threads=1))
    b = flatten(port.run_json(cfg, ds, threads=4))
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_golden_outputs_are_nontrivial():
    for name in CASES:
        _, _, ref = load(name)
        for k, v in ref.items():
            if k.endswith("/real"):
                assert np.abs(v).max() > 0, (name, k)
