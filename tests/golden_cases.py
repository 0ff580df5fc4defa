"""Load the golden fixtures written by ``tests/golden/make_golden.py``.

``CASES`` use the default e-e Pade Jastrow; ``EN_CASES`` use the
electron-nucleus Pade factor, alone ("en") or combined with the e-e factor
("ee+en", CombineJastrow); ``STO_CASES`` use Slater-type orbitals."""
import os

import numpy as np

from qmctorch_gb300.scf import Molecule

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["h2", "lih_cas", "lih_sd", "h2o_sd", "h2o_single", "h4", "c6h6"]
EN_CASES = ["h2_en", "lih_en", "h2o_en", "c6h6_en"]
# Slater-type orbitals in the ADF layout (radial_type "sto", cartesian harmonics)
STO_CASES = ["lih_sto", "h2o_sto"]

_EE = "jastrow.jastrow_terms.0.jastrow_kernel.weight"
_EN = "jastrow.jastrow_terms.1.jastrow_kernel.weight"
_ONLY = "jastrow.jastrow_kernel.weight"


def load(name):
    path = os.path.join(GOLDEN, name + ".npz")
    mol = Molecule(load=path)
    with np.load(path, allow_pickle=False) as f:
        data = {k: f[k] for k in f.files}
    data["configs"] = str(data["case_configs"])
    data["include_all_mo"] = bool(data["case_include_all_mo"])
    data["jastrow"] = str(data["case_jastrow"]) if "case_jastrow" in data else "ee"
    return mol, data


def jastrow_weights(d):
    """[(kind, w)] of the case's Jastrow factors, in the reference's order."""
    if d["jastrow"] == "ee":
        return [("ee", float(d["jastrow_w"][0]))]
    if d["jastrow"] == "en":
        return [("en", float(d["param_" + _ONLY][0]))]
    return [("ee", float(d["param_" + _EE][0])), ("en", float(d["param_" + _EN][0]))]


def param_names(d):
    """State-dict names of the case's Jastrow weights."""
    if d["jastrow"] == "ee" or d["jastrow"] == "en":
        return [_ONLY]
    return [_EE, _EN]


def make_jastrow(mol, d):
    """This package's Jastrow argument of SlaterJastrow for the case."""
    from qmctorch_gb300.wavefunction import (JastrowFactorElectronElectron,
                                             JastrowFactorElectronNuclei, PadeJastrowKernel,
                                             PadeJastrowKernelElectronNuclei)
    if d["jastrow"] == "ee":
        return "default"
    terms = []
    for kind, w in jastrow_weights(d):
        if kind == "ee":
            terms.append(JastrowFactorElectronElectron(mol, PadeJastrowKernel,
                                                       kernel_kwargs={"w": w}))
        else:
            terms.append(JastrowFactorElectronNuclei(mol, PadeJastrowKernelElectronNuclei,
                                                     kernel_kwargs={"w": w}))
    return terms[0] if len(terms) == 1 else terms


def make_wf(mol, d, precision="fp64", cuda=True):
    """SlaterJastrow of the case (configs, MOs, Jastrow factors, CI weights)."""
    import torch
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=cuda,
                       precision=precision, jastrow=make_jastrow(mol, d))
    wf.fc.weight.data = torch.as_tensor(d["fc_weight"], device=wf.fc.weight.device).reshape(1, -1)
    return wf
