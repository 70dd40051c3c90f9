"""The device flux reduction (ffip_flux) on the GPU against the numpy
restatement of Flux_Region / Flux_Box.get_values (ffip/simulation.py:
94-251), on a simulation kept on the device."""
import pytest

from test_flux import check_flux, small_simulation

pytestmark = pytest.mark.gpu


def test_gpu_flux_regions_match_the_reference_restatement():
    import ffip_gb300 as ffip
    freqs = [0.08, 0.1, 0.12]
    sim, box, plane = small_simulation(ffip, freqs)
    sim.run(ffip.run_until_time(120), keep=True)
    try:
        check_flux(ffip, sim, box, plane, freqs)
    finally:
        sim.release()
