"""Loads the golden fixtures (configs + outputs of the reference's own code)."""
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["vacuum_pml", "dispersive", "debye_short", "density_boxes", "pmc_periodic_odd", "pec_periodic_magnetic",
         "decay_stop", "dft_stop"]


def load(name):
    with open(os.path.join(GOLDEN_DIR, name + ".json")) as f:
        d = json.load(f)
    ds = {k: np.asarray(v, dtype=np.float64) for k, v in d["datasets"].items()}
    ref = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    return d["config"], ds, ref


def flatten(out):
    """{group: {name: arr}} -> {"group/name": arr}"""
    return {g + "/" + k: v for g, d in out.items() for k, v in d.items()}
