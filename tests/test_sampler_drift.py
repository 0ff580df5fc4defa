"""CPU tests of the drift-diffusion sampler (GeneralizedMetropolis): its
chains against the reference sampler's own chains on an analytic density
(tests/golden/gmetropolis.npz, written by make_golden.py from the reference
package with the same seed and the same torch CPU generator calls), and the
routing of the drift through a wave function's Jacobi gradient."""
import os

import numpy as np
import torch

from qmctorch_gb300.sampler import GeneralizedMetropolis

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gmetropolis.npz")


def _golden():
    with np.load(GOLDEN) as f:
        return {k: f[k] for k in f.files}


def _density(g):
    a, c = torch.as_tensor(g["a"]), torch.as_tensor(g["c"])
    return lambda x: torch.exp(-(a * (x - c) ** 2).sum(-1)), a, c


def _sampler(g):
    return GeneralizedMetropolis(nwalkers=int(g["cfg_nwalkers"]), nstep=int(g["cfg_nstep"]),
                                 step_size=float(g["cfg_step_size"]),
                                 ntherm=int(g["cfg_ntherm"]), ndecor=int(g["cfg_ndecor"]),
                                 nelec=int(g["cfg_nelec"]), ndim=int(g["cfg_ndim"]),
                                 init={"method": "uniform", "min": -1, "max": 1})


def test_chains_match_the_reference_sampler():
    g = _golden()
    pdf, _, _ = _density(g)
    old = torch.get_default_dtype()
    torch.set_default_dtype(torch.float64)
    try:
        s = _sampler(g)
        torch.manual_seed(int(g["cfg_seed"]))
        out = s(pdf, pos=torch.as_tensor(g["pos0"]), with_tqdm=False)
    finally:
        torch.set_default_dtype(old)
    assert out.requires_grad
    nsnap = (int(g["cfg_nstep"]) - (int(g["cfg_nstep"]) + int(g["cfg_ntherm"])) + 1) // 2
    assert out.shape == g["samples"].shape == (nsnap * int(g["cfg_nwalkers"]), 6)
    np.testing.assert_allclose(out.detach().numpy(), g["samples"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(s.walkers.pos.numpy(), g["final"], rtol=0, atol=1e-12)
    assert not np.allclose(g["final"], g["pos0"])  # the chains moved


class _JacobiDensity(torch.nn.Module):
    """Stands in for a wave function of this package: pdf(x, return_grad=True)
    returns the analytic gradient of the density (the role of the Jacobi
    gradient kernel), and the autograd path is disabled."""

    def __init__(self, a, c):
        super().__init__()
        self.a, self.c = a, c
        self.calls = 0

    def gradients_jacobi(self, x, pdf=False):
        raise AssertionError("not used by the sampler")

    def pdf(self, x, return_grad=False):
        x = x.detach()
        rho = torch.exp(-(self.a * (x - self.c) ** 2).sum(-1))
        if return_grad:
            self.calls += 1
            return -2.0 * self.a * (x - self.c) * rho[:, None]
        return rho


def test_drift_uses_the_wave_function_gradient():
    g = _golden()
    pdf, a, c = _density(g)
    wf = _JacobiDensity(a, c)
    s = _sampler(g)
    x = torch.as_tensor(g["pos0"])
    d_auto = s.get_drift(pdf, x).detach()
    d_jac = s.get_drift(wf.pdf, x)
    assert wf.calls == 1
    np.testing.assert_allclose(d_jac.numpy(), d_auto.numpy(), rtol=1e-12, atol=1e-14)
    # analytic drift grad(rho) / (2 rho) = -a (x - c)
    np.testing.assert_allclose(d_jac.numpy(), (-(a * (x - c))).numpy(), rtol=1e-12, atol=1e-14)
