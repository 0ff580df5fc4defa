"""Hamiltonian Monte Carlo sampler, drop-in for
``qmctorch.sampler.Hamiltonian`` (``qmctorch/sampler/hamiltonian.py:10-201``).

Each step draws Gaussian momenta, runs a leapfrog trajectory of ``L`` steps
of size ``step_size`` on the potential U = -log(pdf), and accepts the end point
with probability min(1, exp(H_start - H_end)) (H = U + |p|^2 / 2). The steps
and the random draws are the reference's (torch's default CPU generator:
momenta, then acceptance uniforms, per step), including what a drop-in must
keep to reproduce its chains:

* every walker is accepted or rejected as a whole (all electrons move);
* the kept positions are those after each step, from ``ntherm`` on, every
  ``ndecor`` steps (hamiltonian.py:113-131).

When ``pdf`` is the bound ``pdf`` of a wave function of this package, the
force -grad U = grad(pdf) / pdf comes from its Jacobi gradient kernel
(``pdf(x, return_grad=True)``, ``qmc_wf_gradients``) and one density call
(``qmc_wf_psi``), instead of autograd through the density; any other callable
is differentiated with autograd as in the reference (get_grad, 40-61). The
trajectory runs on the host: two kernel calls per leapfrog step.
"""
from __future__ import annotations

import logging

import torch

from .metropolis import SamplerBase

log = logging.getLogger("qmctorch_gb300")


class Hamiltonian(SamplerBase):
    """hamiltonian.py:10-38 (same arguments and defaults)."""

    def __init__(self, nwalkers=100, nstep=100, step_size=0.2, L=10, ntherm=-1, ndecor=1,
                 nelec=1, ndim=3, init={"min": -5, "max": 5}, cuda=False):  # noqa: B006
        SamplerBase.__init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim,
                             init, cuda)
        self.traj_length = L

    @staticmethod
    def get_grad(func, inp):
        """grad of ``func`` at ``inp`` by autograd, accumulated into
        ``inp.grad`` as the reference does (hamiltonian.py:40-61)."""
        with torch.enable_grad():
            if inp.grad is not None:
                inp.grad.zero_()
            inp.requires_grad = True
            val = func(inp)
            val.backward(torch.ones(val.shape, dtype=val.dtype, device=val.device))
            inp.requires_grad = False
        return inp.grad

    @staticmethod
    def log_func(func):
        """U = -log(func) (hamiltonian.py:63-73)."""
        return lambda x: -torch.log(func(x))

    @staticmethod
    def _kernel_potential(pdf):
        """(U, grad U) of a wave function's bound pdf by the kernels:
        U = -log pdf, grad U = -grad(pdf) / pdf (Jacobi gradient)."""
        def potential(x):
            return -torch.log(pdf(x))

        def grad(_, x):
            rho = pdf(x).reshape(-1, 1)
            return -pdf(x, return_grad=True) / rho
        return potential, grad

    def __call__(self, pdf, pos=None, with_tqdm=True):
        """Samples after ``ntherm`` steps, every ``ndecor`` steps, concatenated
        over steps (hamiltonian.py:75-131)."""
        if self.ntherm < 0:
            self.ntherm = self.nstep + self.ntherm
        self.walkers.initialize(pos=pos)
        self.walkers.pos = self.walkers.pos.clone()
        owner = getattr(pdf, "__self__", None)
        if owner is not None and hasattr(owner, "gradients_jacobi"):
            potential, grad = self._kernel_potential(pdf)
        else:
            potential, grad = self.log_func(pdf), self.get_grad
        kept, rate, idecor = [], 0.0, 0
        for istep in range(self.nstep):
            self.walkers.pos, r = self._step(potential, grad, self.step_size,
                                             self.traj_length, self.walkers.pos)
            rate += float(r)
            if istep >= self.ntherm:
                if idecor % self.ndecor == 0:
                    kept.append(self.walkers.pos)
                idecor += 1
        log.debug("  Acceptance rate %1.3f %%", rate / max(self.nstep, 1) * 100)
        return torch.cat(kept).requires_grad_()

    @staticmethod
    def _step(U, get_grad, epsilon, L, q_init):
        """One leapfrog trajectory and its accept / reject
        (hamiltonian.py:133-201). Momenta and uniforms are drawn on the CPU
        generator, in the reference's order."""
        q = q_init.clone()
        p = torch.randn(q.shape).to(device=q.device, dtype=q.dtype)
        e_start = U(q) + 0.5 * (p * p).sum(1)
        p -= 0.5 * epsilon * get_grad(U, q)
        for _ in range(L - 1):
            q += epsilon * p
            p -= epsilon * get_grad(U, q)
        q += epsilon * p
        p -= 0.5 * epsilon * get_grad(U, q)
        p = -p
        e_end = U(q) + 0.5 * (p * p).sum(1)
        u = torch.rand(e_end.shape).to(device=e_end.device, dtype=e_end.dtype)
        rejected = torch.exp(e_start - e_end) < u
        q[rejected] = q_init[rejected]
        rate = 1 - rejected.sum().float() / rejected.shape[0]
        return q, rate
