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

When ``pdf`` is the bound ``pdf`` of a wave function of this package (and
``ndim`` is 3), the whole call is one ``qmc_hmc_run`` launch: every walker's
trajectories run on the device, the force -grad U = 2 grad psi / psi from the
Jacobi formula at each leapfrog point. Its random numbers come from the device
generator (Philox, keyed by ``seed`` or by a draw from torch's generator) with
``rng="device"``, the default; with ``rng="torch"`` they are drawn from torch's
CPU generator in the reference's order (momenta, then acceptance uniforms, per
step) and handed to the kernel, so that with the same torch seed the chains are
the reference's. Any other callable runs the host loop, differentiated with
autograd as in the reference (get_grad, 40-61).
"""
from __future__ import annotations

import logging

import torch

from .. import _lib
from ..wavefunction import runtime as rt
from .generalized_metropolis import GeneralizedMetropolis
from .metropolis import SamplerBase

log = logging.getLogger("qmctorch_gb300")


class Hamiltonian(SamplerBase):
    """hamiltonian.py:10-38 (same arguments and defaults)."""

    def __init__(self, nwalkers=100, nstep=100, step_size=0.2, L=10, ntherm=-1, ndecor=1,
                 nelec=1, ndim=3, init={"min": -5, "max": 5}, cuda=False,  # noqa: B006
                 rng="device", seed=None):
        SamplerBase.__init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim,
                             init, cuda)
        self.traj_length = L
        if rng not in ("device", "torch"):
            raise ValueError("rng should be 'device' or 'torch'")
        self.rng = rng
        self._seed = None if seed is None else int(seed)
        self._step_counter = 0
        self.last_acceptance = None

    seed = GeneralizedMetropolis.seed

    def reference_draws(self, nwalkers):
        """The random numbers of one call in the reference's order, from
        torch's default CPU generator: per step the momenta (``_step``'s
        ``torch.randn``) and the acceptance uniforms (``torch.rand``).
        Returns (momenta [nstep, nw, nelec * ndim], uniforms [nstep, nw]), FP64."""
        nc = self.nelec * self.ndim
        mom = torch.empty((self.nstep, nwalkers, nc), dtype=torch.float64)
        unif = torch.empty((self.nstep, nwalkers), dtype=torch.float64)
        for istep in range(self.nstep):
            mom[istep] = torch.randn((nwalkers, nc)).double()
            unif[istep] = torch.rand(nwalkers).double()
        return mom, unif

    def _run_kernel(self, wf):
        """One ``qmc_hmc_run`` launch for the whole call."""
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
        scr = rt.scratch(lib.qmc_hmc_scratch_bytes(call.ref, nw), device)
        a = _lib.HmcArgs()
        a.pos, a.nwalkers, a.nstep = rt.ptr(x), nw, self.nstep
        a.ntherm, a.ndecor, a.traj_length = self.ntherm, self.ndecor, int(self.traj_length)
        a.step_size = float(self.step_size)
        a.samples, a.nsnap, a.accepted = rt.ptr(samples), nsnap, rt.ptr(acc)
        keep = []
        if self.rng == "torch":
            mom, unif = self.reference_draws(nw)
            keep = [mom.to(device), unif.to(device)]
            a.momenta, a.uniforms = rt.ptr(keep[0]), rt.ptr(keep[1])
        else:
            a.seed, a.step_offset = self.seed, self._step_counter
        _lib.check(lib.qmc_hmc_run(call.ref, a, rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   "qmc_hmc_run")
        self._step_counter += self.nstep
        self.last_acceptance = float(acc.sum()) / max(1, nw * self.nstep)
        log.debug("  Acceptance rate %1.3f %%", self.last_acceptance * 100)
        self.walkers.pos = x.to(device=src.device, dtype=src.dtype)
        del keep
        return samples.reshape(nsnap * nw, nc).to(device=src.device,
                                                  dtype=src.dtype).requires_grad_()

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
        wf = GeneralizedMetropolis._wavefunction(pdf)
        if wf is not None and self.ndim == 3:
            with torch.no_grad():
                return self._run_kernel(wf)
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
        self.last_acceptance = rate / max(self.nstep, 1)
        log.debug("  Acceptance rate %1.3f %%", self.last_acceptance * 100)
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
