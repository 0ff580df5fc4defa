"""Calibration of the CPU baseline (test infrastructure, not product code).

The benchmark's CPU baseline times the oracle's numpy restatement of the
reference's Metropolis path (``qmc_oracle.metropolis_replay`` on
``OracleSlaterJastrow.pdf``), because the reference itself cannot be
installed where the benchmark runs. This script times both on the same host
cores and the same workload -- H2O cc-pVDZ, single_double(4,4), Pade e-e
Jastrow, all-electron Gaussian moves of step 0.2 -- one process each with one
thread, and prints walker-steps/s of the reference's own
``Metropolis.__call__`` (qmctorch/sampler/metropolis.py:85-177, FP64 PyTorch)
beside the port's, and their ratio.

Usage (where the reference source tree is available):

    OMP_NUM_THREADS=1 OPENBLAS_NUM_THREADS=1 \\
        python oracle/calibrate_port.py /path/to/QMCTorch [nwalkers] [nstep]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

H2O = "O 0 0 0.1173; H 0 0.7572 -0.4692; H 0 -0.7572 -0.4692"


def main(reference_root, nw=512, nstep=4):
    import ref_stubs
    ref_stubs.install(reference_root)
    import torch
    from qmctorch.sampler import Metropolis
    from qmctorch.utils import set_torch_double_precision
    from qmctorch.wavefunction import SlaterJastrow

    from oracle import qmc_oracle as orc
    from qmctorch_gb300.scf import Molecule

    torch.set_num_threads(1)
    set_torch_double_precision()
    mol = Molecule(H2O, unit="angs", basis="cc-pvdz")
    rng = np.random.default_rng(0)
    centers = np.repeat(np.asarray(mol.atom_coords), mol.atomic_nelec, axis=0)
    pos0 = (centers[None] + rng.normal(size=(nw, mol.nelec, 3))).reshape(nw, -1)
    fc = rng.uniform(size=27)
    # the reference's own sampler on its own wave function
    wf = SlaterJastrow(mol, configs="single_double(4,4)")
    wf.fc.weight.data = torch.as_tensor(fc).reshape(1, -1)
    sampler = Metropolis(nwalkers=nw, nstep=nstep, step_size=0.2, nelec=mol.nelec,
                         init=mol.domain("atomic"))
    sampler(wf.pdf, pos=torch.as_tensor(pos0).clone(), with_tqdm=False)  # warm-up
    t0 = time.perf_counter()
    sampler(wf.pdf, pos=torch.as_tensor(pos0).clone(), with_tqdm=False)
    t_ref = time.perf_counter() - t0
    # the oracle's port on the same walkers
    ow = orc.OracleSlaterJastrow(mol, configs="single_double(4,4)", fc_weight=fc)
    props = rng.normal(size=(nstep, nw, 3 * mol.nelec)) * orc.metropolis_sigma(0.2)
    unif = rng.uniform(size=(nstep, nw))
    orc.metropolis_replay(ow.pdf, pos0, props[:1], unif[:1])  # warm-up
    t0 = time.perf_counter()
    orc.metropolis_replay(ow.pdf, pos0, props, unif)
    t_port = time.perf_counter() - t0
    ref_rate, port_rate = nw * nstep / t_ref, nw * nstep / t_port
    return {"workload": "h2o_ccpvdz_single_double44", "nwalkers": nw, "nstep": nstep,
            "threads": 1, "torch": torch.__version__, "numpy": np.__version__,
            "reference_walker_steps_per_s": ref_rate, "port_walker_steps_per_s": port_rate,
            "port_over_reference": port_rate / ref_rate}


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: calibrate_port.py REFERENCE_ROOT [nwalkers] [nstep]")
    args = [int(a) for a in sys.argv[2:4]]
    print(json.dumps(main(sys.argv[1], *args)))
