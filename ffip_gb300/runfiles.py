"""Run files of the run_sim_json driver (ffip_gb300/_lib/run_sim_json):
config.json plus the input datasets, and the outputs it writes.

The reference keeps both in HDF5 (input.h5 with one dataset per name,
output.h5 with one group per monitor; src/simulation.cpp:151-157,
src/dft.cpp:273-320).  Here they are directories of .npy files beside the
named file: <input file>.d/<dataset>.npy and
<fields output file>.d/<group>/<array>.npy.  With h5py installed,
`to_hdf5` / `from_hdf5` convert a directory to or from the reference's HDF5
layout."""
from __future__ import annotations

import json
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(HERE, "_lib", "run_sim_json")


def write_inputs(directory: str, config: dict, datasets: Optional[Dict[str, np.ndarray]] = None) -> str:
    """Writes config.json and the input datasets into `directory`."""
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "config.json"), "w") as f:
        json.dump(config, f, indent=4)
    ds_dir = os.path.join(directory, config.get("input file", "input.h5") + ".d")
    os.makedirs(ds_dir, exist_ok=True)
    for name, v in (datasets or {}).items():
        np.save(os.path.join(ds_dir, name + ".npy"), np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel()))
    return directory


def read_outputs(directory: str, config: dict) -> Dict[str, Dict[str, np.ndarray]]:
    """The output groups the driver wrote, as {group: {array: ndarray}}."""
    out_dir = os.path.join(directory, config.get("fields output file", "output.h5") + ".d")
    res = {}
    for g in sorted(os.listdir(out_dir)):
        gdir = os.path.join(out_dir, g)
        res[g] = {a[:-4]: np.load(os.path.join(gdir, a)) for a in sorted(os.listdir(gdir)) if a.endswith(".npy")}
    return res


def run(directory: str, exe: Optional[str] = None, timeout: Optional[float] = None) -> subprocess.CompletedProcess:
    """Runs the driver in `directory` (it reads ./config.json there)."""
    return subprocess.run([exe or CLI], cwd=directory, capture_output=True, text=True, timeout=timeout)


def to_hdf5(npy_dir: str, h5_path: str):
    """Copies a .npy directory (datasets, or groups of datasets) into an HDF5 file."""
    import h5py
    with h5py.File(h5_path, "w") as f:
        for name in sorted(os.listdir(npy_dir)):
            p = os.path.join(npy_dir, name)
            if os.path.isdir(p):
                grp = f.create_group(name)
                for a in sorted(os.listdir(p)):
                    grp.create_dataset(a[:-4], data=np.load(os.path.join(p, a)))
            elif name.endswith(".npy"):
                f.create_dataset(name[:-4], data=np.load(p))


def from_hdf5(h5_path: str, npy_dir: str):
    """Copies the datasets (and groups of datasets) of an HDF5 file into a .npy directory."""
    import h5py
    os.makedirs(npy_dir, exist_ok=True)
    with h5py.File(h5_path, "r") as f:
        for name, item in f.items():
            if isinstance(item, h5py.Group):
                os.makedirs(os.path.join(npy_dir, name), exist_ok=True)
                for a, d in item.items():
                    np.save(os.path.join(npy_dir, name, a + ".npy"), np.asarray(d))
            else:
                np.save(os.path.join(npy_dir, name + ".npy"), np.asarray(item).ravel())
