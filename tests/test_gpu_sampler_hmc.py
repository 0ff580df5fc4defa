"""HMC on an H2 sto-3g SlaterJastrow of this package, forces from the Jacobi
gradient kernel (qmc_wf_gradients) and densities from the psi kernel, against
the reference sampler's chains on its own H2 wave function with autograd
forces (tests/golden/hamiltonian.npz), same seed and initial walkers. The
forces agree to rounding (the Jacobi gradient equals the autograd gradient to
~1e-15), so 12 steps of 6 leapfrog steps stay within 1e-9."""
import numpy as np
import pytest
import torch

from tests.golden_cases import GOLDEN, load

pytestmark = pytest.mark.gpu

HMC = {"nwalkers": 16, "nelec": 2, "ndim": 3, "nstep": 12, "step_size": 0.1, "L": 6,
       "ntherm": -6, "ndecor": 2, "seed": 777}


def test_hmc_chains_match_reference_on_h2():
    import os

    from qmctorch_gb300.sampler import Hamiltonian
    from qmctorch_gb300.wavefunction import SlaterJastrow
    torch.set_default_dtype(torch.float64)
    with np.load(os.path.join(GOLDEN, "hamiltonian.npz")) as f:
        gold = {k: f[k] for k in f.files}
    mol, d = load("h2")
    wf = SlaterJastrow(mol, configs="ground_state", include_all_mo=True, cuda=True)
    g = HMC
    s = Hamiltonian(nwalkers=g["nwalkers"], nstep=g["nstep"], step_size=g["step_size"], L=g["L"],
                    ntherm=g["ntherm"], ndecor=g["ndecor"], nelec=g["nelec"], ndim=g["ndim"],
                    init={"method": "uniform", "min": -1, "max": 1}, cuda=True)
    torch.manual_seed(g["seed"] + 1)
    out = s(wf.pdf, pos=torch.as_tensor(gold["h2_pos0"], device="cuda"), with_tqdm=False)
    np.testing.assert_allclose(out.detach().cpu().numpy(), gold["h2_samples"], rtol=1e-9,
                               atol=1e-9)
