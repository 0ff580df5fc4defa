"""Drift-diffusion (generalized) Metropolis sampler, drop-in for
``qmctorch.sampler.GeneralizedMetropolis``
(``qmctorch/sampler/generalized_metropolis.py:12-219``).

Each step moves one randomly chosen electron per walker by
``step * drift + N(0, sqrt(step) I)``, with the drift ``grad(rho) / (2 rho)`` of
the sampled density, and accepts with the ratio of the transition kernels times
the density ratio. The steps follow the reference, including what a drop-in
must keep to reproduce its chains:

* proposals start from the walkers' positions at the start of the call (the
  reference reads ``walkers.pos``, which it writes back only after the last
  step; generalized_metropolis.py:133-134, 117);
* the proposal covariance is ``sqrt(step_size) * I`` (150-155) and the
  transition kernel ``exp(-|x_f - x_i - step drift_i| / (2 step))`` uses the
  norm of the whole walker vector, not its square (176-177);
* random draws come from torch's default CPU generator in the reference's
  order per step: electron indices, proposal normals, acceptance uniforms.

When ``pdf`` is the bound ``pdf`` of a wave function of this package, the
drift comes from its Jacobi gradient (``pdf(x, return_grad=True)``: the
``qmc_wf_gradients`` kernel) instead of autograd through the density; any other
callable is differentiated with autograd as in the reference (get_drift,
180-197). The loop runs on the host: two kernel calls per step (density and
gradient), which bounds it by launch latency for small walker counts.
"""
from __future__ import annotations

import logging

import numpy as np
import torch
from torch.distributions import MultivariateNormal

from .metropolis import SamplerBase

log = logging.getLogger("qmctorch_gb300")


class GeneralizedMetropolis(SamplerBase):
    """generalized_metropolis.py:12-44 (same arguments and defaults)."""

    def __init__(self, nwalkers=100, nstep=1000, step_size=3, ntherm=-1, ndecor=1, nelec=1,
                 ndim=1, init={"type": "uniform", "min": -5, "max": 5},  # noqa: B006
                 cuda=False):
        SamplerBase.__init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim,
                             init, cuda)

    def __call__(self, pdf, pos=None, with_tqdm=True):
        """Samples of ``pdf`` after ``ntherm`` steps, every ``ndecor`` steps,
        concatenated over steps: ``(nsnap * nwalkers, nelec * ndim)``
        (generalized_metropolis.py:46-123)."""
        with torch.no_grad():
            if self.ntherm < 0:
                self.ntherm = self.nstep + self.ntherm
            self.walkers.initialize(pos=pos)
            xi = self.walkers.pos.clone()
            rhoi = pdf(xi)
            drifti = self.get_drift(pdf, xi, rho=rhoi)
            rhoi[rhoi == 0] = 1e-16
            out, rate, idecor = [], 0.0, 0
            for istep in range(self.nstep):
                xf = self.move(drifti)
                rhof = pdf(xf)
                driftf = self.get_drift(pdf, xf, rho=rhof)
                rhof[rhof == 0.0] = 1e-16
                tif = self.trans(xi, xf, driftf)
                tfi = self.trans(xf, xi, drifti)
                pmat = (tif * rhof) / (tfi * rhoi).double()
                index = self._accept(pmat)
                rate += float(index.sum()) / self.walkers.nwalkers
                xi[index, :] = xf[index, :]
                rhoi[index] = rhof[index]
                rhoi[rhoi == 0] = 1e-16
                drifti[index, :] = driftf[index, :]
                if istep >= self.ntherm:
                    if idecor % self.ndecor == 0:
                        out.append(xi.clone().detach())
                    idecor += 1
            log.debug("  Acceptance rate %1.3f", rate / max(self.nstep, 1) * 100)
            self.walkers.pos.data = xi.data
        return torch.cat(out).requires_grad_()

    def move(self, drift):
        """Move one random electron per walker (generalized_metropolis.py:125-143):
        from the walkers' positions at the start of the call."""
        nw = self.walkers.nwalkers
        new_pos = self.walkers.pos.clone().view(nw, self.nelec, self.ndim)
        index = torch.LongTensor(nw).random_(0, self.nelec)  # CPU generator, as the reference
        step = self._move(drift, index)
        rows = torch.arange(nw)
        dev = new_pos.device
        new_pos[rows.to(dev), index.to(dev), :] += step.to(device=dev, dtype=new_pos.dtype)
        return new_pos.view(nw, self.nelec * self.ndim)

    def _move(self, drift, index):
        """step * drift of the moved electron + N(0, sqrt(step) I)
        (generalized_metropolis.py:145-167)."""
        nw = self.walkers.nwalkers
        d = drift.view(nw, self.nelec, self.ndim)
        mv = MultivariateNormal(torch.zeros(self.ndim), np.sqrt(self.step_size) * torch.eye(self.ndim))
        noise = mv.sample((nw, 1)).squeeze()  # CPU generator, after the electron indices
        moved = d[torch.arange(nw, device=d.device), index.to(d.device), :]
        return self.step_size * moved + noise.to(device=d.device, dtype=d.dtype)

    def trans(self, xf, xi, drifti):
        """exp(-|xf - xi - step drifti| / (2 step)) per walker
        (generalized_metropolis.py:169-177)."""
        a = (xf - xi - drifti * self.step_size).norm(dim=1)
        return torch.exp(-0.5 * a / self.step_size)

    def get_drift(self, pdf, x, rho=None):
        """grad(rho) / (2 rho) (generalized_metropolis.py:180-197): by the
        wave function's Jacobi gradient kernel when ``pdf`` is the bound pdf
        of a wave function of this package, else by autograd. ``rho`` = pdf(x)
        when the caller has it already (the Jacobi path then makes one kernel
        call, the gradient)."""
        owner = getattr(pdf, "__self__", None)
        if owner is not None and hasattr(owner, "gradients_jacobi"):
            if rho is None:
                rho = pdf(x)
            grad_rho = pdf(x, return_grad=True)
            return 0.5 * grad_rho / rho.view(-1, 1)
        with torch.enable_grad():
            xg = x.detach().requires_grad_(True)
            rho = pdf(xg).view(-1, 1)
            grad_rho = torch.autograd.grad(rho, xg, grad_outputs=torch.ones_like(rho))[0]
            return 0.5 * grad_rho / rho

    def _accept(self, P):
        """min(1, P) - u >= 0, u ~ U(0,1) from the CPU generator
        (generalized_metropolis.py:199-219)."""
        P[P > 1] = 1.0
        tau = torch.rand(self.walkers.nwalkers, dtype=torch.float64)
        return (P - tau.to(P.device) >= 0).reshape(-1).type(torch.bool)
