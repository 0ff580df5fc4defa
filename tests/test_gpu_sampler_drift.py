"""GPU test of the drift-diffusion sampler on a wave function of this
package: its chains, with the drift from the Jacobi gradient kernel
(qmc_wf_gradients) and the density from qmc_wf_psi, against the chains of the
reference's GeneralizedMetropolis on its own H2 sto-3g SlaterJastrow (autograd
drift), same seed and initial walkers (tests/golden/gmetropolis.npz).
Tolerance: 1e-9 absolute on the positions (FP64 density and drift agree with
the reference's to about 1e-14; the accept / reject decisions are the same)."""
import os

import numpy as np
import pytest
import torch

from tests.golden_cases import load

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gmetropolis.npz")


def test_drift_sampler_chains_match_the_reference_on_h2():
    from qmctorch_gb300.sampler import GeneralizedMetropolis
    from qmctorch_gb300.wavefunction import SlaterJastrow
    with np.load(GOLDEN) as f:
        g = {k: f[k] for k in f.files}
    torch.set_default_dtype(torch.float64)
    mol, d = load("h2")
    wf = SlaterJastrow(mol, configs=d["configs"], include_all_mo=d["include_all_mo"], cuda=True)
    s = GeneralizedMetropolis(nwalkers=16, nstep=20, step_size=0.2, ntherm=-10, ndecor=2,
                              nelec=mol.nelec, ndim=3, cuda=True,
                              init={"method": "uniform", "min": -1, "max": 1})
    torch.manual_seed(int(g["cfg_seed"]) + 1)
    out = s(wf.pdf, pos=torch.as_tensor(g["h2_pos0"], device="cuda"), with_tqdm=False)
    assert out.is_cuda and out.shape == g["h2_samples"].shape
    np.testing.assert_allclose(out.detach().cpu().numpy(), g["h2_samples"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(s.walkers.pos.cpu().numpy(), g["h2_final"], rtol=0, atol=1e-9)
