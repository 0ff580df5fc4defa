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

When ``pdf`` is the bound ``pdf`` of a wave function of this package (and
``ndim`` is 3), the whole call is one ``qmc_drift_run`` launch: every walker's
steps run on the device, with psi and the drift grad psi / psi from the Jacobi
formula at each proposal. Its random numbers come from the device generator
(Philox, keyed by ``seed`` or by a draw from torch's generator) with
``rng="device"``, the default; with ``rng="torch"`` they are drawn from torch's
default CPU generator in the reference's order and handed to the kernel, so
that with the same torch seed the chains are the reference's. Any other
callable runs the host loop, its drift differentiated with autograd as in the
reference (get_drift, 180-197).
"""
from __future__ import annotations

import logging

import numpy as np
import torch
from torch.distributions import MultivariateNormal

from .. import _lib
from ..wavefunction import runtime as rt
from .metropolis import SamplerBase

log = logging.getLogger("qmctorch_gb300")


class GeneralizedMetropolis(SamplerBase):
    """generalized_metropolis.py:12-44 (same arguments and defaults)."""

    def __init__(self, nwalkers=100, nstep=1000, step_size=3, ntherm=-1, ndecor=1, nelec=1,
                 ndim=1, init={"type": "uniform", "min": -5, "max": 5},  # noqa: B006
                 cuda=False, rng="device", seed=None):
        SamplerBase.__init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim,
                             init, cuda)
        if rng not in ("device", "torch"):
            raise ValueError("rng should be 'device' or 'torch'")
        self.rng = rng
        self._seed = None if seed is None else int(seed)
        self._step_counter = 0
        self.last_acceptance = None

    @property
    def seed(self):
        """Key of the kernel's generator (``rng="device"``): the ``seed``
        argument, else drawn from torch's generator at the first launch."""
        if self._seed is None:
            self._seed = int(torch.randint(0, 2 ** 62, (1,)).item())
        return self._seed

    @seed.setter
    def seed(self, value):
        self._seed = int(value)

    def __call__(self, pdf, pos=None, with_tqdm=True):
        """Samples of ``pdf`` after ``ntherm`` steps, every ``ndecor`` steps,
        concatenated over steps: ``(nsnap * nwalkers, nelec * ndim)``
        (generalized_metropolis.py:46-123)."""
        with torch.no_grad():
            if self.ntherm < 0:
                self.ntherm = self.nstep + self.ntherm
            self.walkers.initialize(pos=pos)
            wf = self._wavefunction(pdf)
            if wf is not None:
                return self._run_kernel(wf)
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
            self.last_acceptance = rate / max(self.nstep, 1)
            log.debug("  Acceptance rate %1.3f", self.last_acceptance * 100)
            self.walkers.pos.data = xi.data
        return torch.cat(out).requires_grad_()

    @staticmethod
    def _wavefunction(pdf):
        """The wave function of this package whose bound ``pdf`` this is, or None."""
        from ..wavefunction.slater_jastrow import SlaterJastrow
        wf = getattr(pdf, "__self__", None)
        if isinstance(wf, SlaterJastrow) and getattr(pdf, "__name__", "") == "pdf":
            return wf
        return None

    def reference_draws(self, nwalkers):
        """The random numbers of one call in the reference's order, from
        torch's default CPU generator: per step the moved electrons
        (``move``), the proposal noise (``_move``) and the acceptance
        uniforms (``_accept``). Returns (electron index [nstep, nw] int32,
        noise [nstep, nw, 3], uniforms [nstep, nw]) in FP64."""
        idx = torch.empty((self.nstep, nwalkers), dtype=torch.int32)
        noise = torch.empty((self.nstep, nwalkers, self.ndim), dtype=torch.float64)
        tau = torch.empty((self.nstep, nwalkers), dtype=torch.float64)
        for istep in range(self.nstep):
            idx[istep] = torch.LongTensor(nwalkers).random_(0, self.nelec).to(torch.int32)
            mv = MultivariateNormal(torch.zeros(self.ndim),
                                    np.sqrt(self.step_size) * torch.eye(self.ndim))
            noise[istep] = mv.sample((nwalkers, 1)).reshape(nwalkers, self.ndim).double()
            tau[istep] = torch.rand(nwalkers, dtype=torch.float64)
        return idx, noise, tau

    def _run_kernel(self, wf):
        """One ``qmc_drift_run`` launch for the whole call; the walkers'
        final positions are written back as the reference does."""
        if self.ndim != 3:
            raise ValueError("a wave function of this package is sampled in 3 dimensions")
        nsnap = len(range(self.ntherm, self.nstep, self.ndecor))
        if nsnap == 0:
            raise RuntimeError("no samples kept: ntherm >= nstep")
        device = rt.cuda_device()
        src = self.walkers.pos.detach()
        x = rt.dev64(src, device)
        if x.data_ptr() == src.data_ptr():
            x = x.clone()
        nw = x.shape[0]
        nc = self.nelec * self.ndim
        samples = torch.empty((nsnap, nw, nc), dtype=rt.F64, device=device)
        acc = torch.zeros(nw, dtype=torch.int32, device=device)
        call = wf._desc(device)
        lib = _lib.lib()
        scr = rt.scratch(lib.qmc_drift_scratch_bytes(call.ref, nw), device)
        a = _lib.DriftArgs()
        a.pos, a.nwalkers, a.nstep = rt.ptr(x), nw, self.nstep
        a.ntherm, a.ndecor, a.step_size = self.ntherm, self.ndecor, float(self.step_size)
        a.samples, a.nsnap, a.accepted = rt.ptr(samples), nsnap, rt.ptr(acc)
        keep = []
        if self.rng == "torch":
            idx, noise, tau = self.reference_draws(nw)
            keep = [idx.to(device), noise.to(device), tau.to(device)]
            a.electron_index, a.normals, a.uniforms = (rt.ptr(t) for t in keep)
        else:
            a.seed, a.step_offset = self.seed, self._step_counter
        _lib.check(lib.qmc_drift_run(call.ref, a, rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   "qmc_drift_run")
        self._step_counter += self.nstep
        self.last_acceptance = float(acc.sum()) / max(1, nw * self.nstep)
        log.debug("  Acceptance rate %1.3f", self.last_acceptance * 100)
        self.walkers.pos.data = x.to(device=src.device, dtype=src.dtype)
        out = samples.reshape(nsnap * nw, nc).to(device=src.device, dtype=src.dtype)
        del keep
        return out.requires_grad_()

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
