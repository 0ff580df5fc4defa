"""Load the golden fixtures written by ``tests/golden/make_golden.py``."""
import os

import numpy as np

from qmctorch_gb300.scf import Molecule

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["h2", "lih_cas", "lih_sd", "h2o_sd", "h2o_single", "h4", "c6h6"]


def load(name):
    path = os.path.join(GOLDEN, name + ".npz")
    mol = Molecule(load=path)
    with np.load(path, allow_pickle=False) as f:
        data = {k: f[k] for k in f.files}
    data["configs"] = str(data["case_configs"])
    data["include_all_mo"] = bool(data["case_include_all_mo"])
    return mol, data
