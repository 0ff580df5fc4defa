"""Metropolis sampler (drop-in for ``qmctorch.sampler.Metropolis``,
``qmctorch/sampler/metropolis.py:10-298``) and walkers
(``qmctorch/sampler/walkers.py:8-150``).

Sampling a wave function of this package runs ``qmc_metropolis_run``: one
persistent launch in which each thread advances one walker chain through all
steps (proposal, psi re-evaluation, accept/reject, snapshot), with a Philox
counter-based generator seeded per sampler. Walker initialisation mirrors the
reference's host-side RNG calls, so a seeded initial configuration is the
reference's.

Any other density callable (an analytic pdf, a user model) is sampled by the
reference's own algorithm as a host loop of torch operations on the walkers'
device, with the reference's random draws (torch's generators, in its order),
so that a seeded chain is the reference's chain.
"""
from __future__ import annotations

import logging
import time

import numpy as np
import torch
from torch.distributions import MultivariateNormal

from .. import _lib
from ..wavefunction import runtime as rt

log = logging.getLogger("qmctorch_gb300")

_PINNED_OUT_MAX = 256 << 20  # largest host result returned in page-locked memory (bytes)
_MOVE = {"all-elec": 0, "one-elec": 1, "all-elec-iter": 2}
_PROBA = {"normal": 0, "uniform": 1}


class Walkers:
    """Walker positions and their initialisation (walkers.py:8-150)."""

    def __init__(self, nwalkers=100, nelec=1, ndim=3, init=None, cuda=False):
        self.nwalkers = nwalkers
        self.ndim = ndim
        self.nelec = nelec
        self.init_domain = init
        self.pos = None
        self.status = None
        self.cuda = cuda
        self.device = torch.device("cuda") if cuda else torch.device("cpu")

    def initialize(self, pos=None):
        if pos is not None:
            if len(pos) > self.nwalkers:
                pos = pos[-self.nwalkers:, :]
            self.pos = pos
            return
        if "center" in self.init_domain:
            self.pos = self._init_center()
        elif "min" in self.init_domain:
            self.pos = self._init_uniform()
        elif "mean" in self.init_domain:
            self.pos = self._init_multivar()
        elif "atom_coords" in self.init_domain:
            self.pos = self._init_atomic()
        else:
            raise ValueError("Init walkers not recognized")

    def _init_center(self):
        eps = 1e-3
        pos = -eps + 2 * eps * torch.rand(self.nwalkers, self.nelec * self.ndim)
        return pos.type(torch.get_default_dtype()).to(device=self.device)

    def _init_uniform(self):
        pos = torch.rand(self.nwalkers, self.nelec * self.ndim)
        pos *= self.init_domain["max"] - self.init_domain["min"]
        pos += self.init_domain["min"]
        return pos.type(torch.get_default_dtype()).to(device=self.device)

    def _init_multivar(self):
        multi = MultivariateNormal(torch.as_tensor(self.init_domain["mean"]),
                                   torch.as_tensor(self.init_domain["sigma"]))
        pos = multi.sample((self.nwalkers, self.nelec)).type(torch.get_default_dtype())
        return pos.view(self.nwalkers, self.nelec * self.ndim).to(device=self.device)

    def _init_atomic(self):
        pos = torch.zeros(self.nwalkers, self.nelec * self.ndim)
        idx_ref, nelec_tot, natom = [], 0, 0
        for iat, ne in enumerate(self.init_domain["atom_nelec"]):
            idx_ref += [iat] * ne
            nelec_tot += ne
            natom += 1
        for iw in range(self.nwalkers):
            placed = [0] * natom
            idx = torch.as_tensor(idx_ref)[torch.randperm(nelec_tot)]
            xyz = torch.as_tensor(self.init_domain["atom_coords"])[idx, :]
            for ie in range(nelec_tot):
                i = idx[ie]
                if placed[i] == 0:
                    s = 1.0 / self.init_domain["atom_num"][i]
                elif placed[i] < 5:
                    s = 2.0 / (self.init_domain["atom_num"][i] - 2)
                else:
                    s = 3.0 / (self.init_domain["atom_num"][i] - 3)
                xyz[ie, :] += torch.as_tensor(np.random.normal(scale=s, size=(1, 3)),
                                              dtype=xyz.dtype).reshape(3)
                placed[i] += 1
            pos[iw, :] = xyz.view(-1)
        return pos.to(device=self.device)


class SamplerBase:
    """sampler_base.py:7-91."""

    def __init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim, init, cuda):
        self.nelec = nelec
        self.ndim = ndim
        self.nstep = nstep
        self.step_size = step_size
        self.ntherm = ntherm
        self.ndecor = ndecor
        self.cuda = cuda
        self.device = torch.device("cuda") if cuda else torch.device("cpu")
        self.walkers = Walkers(nwalkers=nwalkers, nelec=nelec, ndim=ndim, init=init, cuda=cuda)

    def __repr__(self):
        return self.__class__.__name__ + " sampler with  %d walkers" % self.walkers.nwalkers

    def get_sampling_size(self):
        if self.ntherm == -1:
            return self.walkers.nwalkers
        return self.walkers.nwalkers * int((self.nstep - self.ntherm) / self.ndecor)


class Metropolis(SamplerBase):
    """metropolis.py:10-298. ``logspace=True`` selects the reference's test
    ``min(0, log rho' - log rho) - log u >= 0`` (288-292), the same acceptance
    rule as ``min(1, rho' / rho) - u >= 0`` up to rounding at the boundary; the
    kernel evaluates the ratio form for both settings."""

    def __init__(self, nwalkers=100, nstep=1000, step_size=0.2, ntherm=-1, ndecor=1, nelec=1,
                 ndim=3, init={"min": -5, "max": 5}, move={"type": "all-elec", "proba": "normal"},
                 logspace=False, symmetry=None, cuda=False, seed=None):
        SamplerBase.__init__(self, nwalkers, nstep, step_size, ntherm, ndecor, nelec, ndim, init,
                             cuda)
        self.logspace = logspace
        self.configure_move(move)
        self.symmetry = (lambda x: x) if symmetry is None else symmetry
        self._seed = None if seed is None else int(seed)
        self._step_counter = 0
        self.last_acceptance = None

    @property
    def seed(self):
        """Key of the kernel's Philox generator. Without a ``seed`` argument it
        is drawn from torch's generator at the first kernel launch, not at
        construction, so that building a sampler draws nothing (the host loop
        of an arbitrary density then sees torch's generator as the reference
        does)."""
        if self._seed is None:
            self._seed = int(torch.randint(0, 2 ** 62, (1,)).item())
        return self._seed

    @seed.setter
    def seed(self, value):
        self._seed = int(value)

    def configure_move(self, move):
        """metropolis.py:179-225."""
        self.movedict = move
        if "type" not in self.movedict:
            self.movedict["type"] = "one-elec"
        if "proba" not in self.movedict:
            self.movedict["proba"] = "uniform"
        if self.movedict["type"] not in _MOVE:
            raise ValueError(" 'type' in move should be 'one-elec','all-elec', 'all-elec-iter'")
        if self.movedict["proba"] not in _PROBA:
            raise ValueError("'proba' in move should be 'normal' or 'uniform'")
        self._move_per_iter = self.nelec if self.movedict["type"] == "all-elec-iter" else 1
        self.fixed_id_elec_list = (range(self.nelec) if self.movedict["type"] == "all-elec-iter"
                                   else [None])
        # proposal law of the host loop (a construction draws nothing)
        self._normal = None
        if self.movedict["proba"] == "normal":
            var = self.step_size / (2 * torch.sqrt(2 * torch.log(torch.as_tensor(2.0))))
            self._normal = MultivariateNormal(torch.zeros(self.ndim), var * torch.eye(self.ndim))

    def _wavefunction(self, pdf, required=True):
        """The wave function whose bound ``pdf`` this is, or None (or
        TypeError when ``required``) for any other callable."""
        wf = getattr(pdf, "__self__", None)
        from ..wavefunction.slater_jastrow import SlaterJastrow
        if not isinstance(wf, SlaterJastrow) or getattr(pdf, "__name__", "") != "pdf":
            if required:
                raise TypeError("device-resident sampling needs the pdf of a qmctorch_gb300 "
                                "wave function: pass wf.pdf")
            return None
        return wf

    def nsnap(self):
        ntherm = self.ntherm if self.ntherm >= 0 else self.nstep + self.ntherm
        return len(range(ntherm, self.nstep, self.ndecor))

    def _run_kernel(self, wf, x, device, samples=None, nsnap=0, accepted=None, replay=None,
                    nstep=None, ntherm=None, scratch=None):
        """One ``qmc_metropolis_run`` launch on the current stream; ``x``
        (nw, 3*nelec) FP64 on ``device`` is advanced in place."""
        nw = x.shape[0]
        call = wf._desc(device)
        lib = _lib.lib()
        need = lib.qmc_metropolis_scratch_bytes(call.ref, nw)
        scr = scratch if (scratch is not None and scratch.numel() >= need) else rt.scratch(need,
                                                                                         device)
        nstep = self.nstep if nstep is None else nstep
        a = _lib.MetropolisArgs()
        a.pos = rt.ptr(x)
        a.nwalkers = nw
        a.nstep = nstep
        a.ntherm = (self.ntherm if ntherm is None else ntherm)
        a.ndecor = self.ndecor
        a.move_type = _MOVE[self.movedict["type"]]
        a.proba = _PROBA[self.movedict["proba"]]
        a.step_size = float(self.step_size)
        a.seed = self.seed
        a.step_offset = self._step_counter
        a.samples = rt.ptr(samples)
        a.nsnap = nsnap
        a.accepted = rt.ptr(accepted)
        a.psi_out = None
        keep = [scr]
        if replay is not None:
            props = rt.dev64(replay["proposals"], device)
            unif = rt.dev64(replay["uniforms"], device)
            keep += [props, unif]
            a.proposals, a.uniforms = rt.ptr(props), rt.ptr(unif)
            if replay.get("electron_index") is not None:
                ei = torch.as_tensor(replay["electron_index"]).to(device, torch.int32).contiguous()
                keep.append(ei)
                a.electron_index = rt.ptr(ei)
        _lib.check(lib.qmc_metropolis_run(call.ref, a, rt.ptr(scr), scr.numel(),
                                          rt.stream_handle()), "qmc_metropolis_run")
        return keep

    def advance(self, pdf, x, nstep=None, accepted=None, scratch=None):
        """Device-resident sampling: advance the walkers ``x`` (CUDA FP64,
        (nw, 3*nelec)) by ``nstep`` Metropolis steps in place, keeping no
        snapshots. Launches exactly one kernel."""
        wf = self._wavefunction(pdf)
        nstep = self.nstep if nstep is None else nstep
        keep = self._run_kernel(wf, x, x.device, accepted=accepted, nstep=nstep, ntherm=nstep,
                                scratch=scratch)
        self._step_counter += nstep
        return keep

    def __call__(self, pdf, pos=None, with_tqdm=True, replay=None):
        """Sample ``pdf`` (= wf.pdf); returns the kept positions
        (nsnap * nwalkers, 3 * nelec) (metropolis.py:85-177).

        ``replay`` (tests) = dict(proposals=..., uniforms=..., electron_index=...)
        replaces the generator with the caller's random numbers, in the
        layouts of ``qmc_metropolis_args``. A ``pdf`` that is not a wave
        function of this package is sampled by the host loop
        (:meth:`_sample_density`)."""
        wf = self._wavefunction(pdf, required=False)
        if wf is None:
            if replay is not None:
                raise ValueError("replay inputs apply to the wave-function kernel only")
            return self._sample_density(pdf, pos, with_tqdm)
        if self.ntherm >= self.nstep:
            raise ValueError("Thermalisation longer than trajectory")
        if self.ntherm < 0:
            self.ntherm = self.nstep + self.ntherm
        device = rt.cuda_device()
        out_device = pos.device if pos is not None else (
            torch.device("cuda") if self.cuda else torch.device("cpu"))
        out_dtype = pos.dtype if pos is not None else torch.get_default_dtype()
        with torch.no_grad():
            self.walkers.initialize(pos=pos)
            src = self.walkers.pos.detach()
            if (src.device.type == "cpu" and src.is_pinned() and src.dtype == rt.F64
                    and src.is_contiguous()):
                # page-locked host walkers: an asynchronous DMA, ordered before
                # the kernel on the same stream
                x = torch.empty(src.shape, dtype=rt.F64, device=device)
                x.copy_(src, non_blocking=True)
            else:
                x = rt.dev64(src, device)
                if x.data_ptr() == src.data_ptr():
                    x = x.clone()  # the walkers are written back below, not in the kernel
            nw = x.shape[0]
            nsnap = len(range(self.ntherm, self.nstep, self.ndecor))
            samples = torch.empty((max(nsnap, 1), nw, self.nelec * self.ndim), dtype=rt.F64,
                                  device=device)
            acc = torch.zeros(nw, dtype=torch.int32, device=device)
            tstart = time.time()
            self._run_kernel(wf, x, device, samples=samples, nsnap=nsnap, accepted=acc,
                             replay=replay)
            self._step_counter += self.nstep
            # the reference updates the walker tensor (and so a caller's pos) in place;
            # copy_ from the device writes a pinned host tensor by DMA, without a
            # pageable staging copy
            out = samples[:nsnap].reshape(nsnap * nw, -1)
            pinned_out = (out_device.type == "cpu"
                          and 0 < out.numel() * out.element_size() <= _PINNED_OUT_MAX)
            wp = self.walkers.pos
            if wp.shape == x.shape:
                # into page-locked memory the copy need not wait here when the
                # result copy below synchronises the stream
                wp.data.copy_(x if wp.dtype == x.dtype else x.to(dtype=wp.dtype),
                              non_blocking=pinned_out and wp.is_pinned())
            else:
                self.walkers.pos = x.to(device=wp.device, dtype=out_dtype)
            if with_tqdm:
                rate = float(acc.sum()) / (nw * self._move_per_iter * self.nstep)
                self.last_acceptance = rate
                dt = time.time() - tstart
                log.info("   Acceptance rate     : %1.2f %%", rate * 100)
                log.info("   Timing statistics   : %1.2f steps/sec.", self.nstep / dt)
                log.info("   Total Time          : %1.2f sec.", dt)
            self._last_accepted = acc
            if pinned_out:
                # host result in page-locked memory (the host allocator caches it):
                # one DMA instead of a staged copy
                host = torch.empty(out.shape, dtype=out_dtype, pin_memory=True)
                host.copy_(out if out.dtype == out_dtype else out.to(dtype=out_dtype))
                out = host
        out = out.to(device=out_device, dtype=out_dtype)
        return self.symmetry(out).requires_grad_()

    # ------------------------------------------------------------------
    # host loop for an arbitrary density (metropolis.py:85-298)
    # ------------------------------------------------------------------
    def _sample_density(self, pdf, pos, with_tqdm):
        """Metropolis chain of any callable ``pdf`` (positions -> density) on
        the walkers' device: proposals, density calls and acceptance as the
        reference takes them, including its random draws, so that with the
        same torch seed the chain is the reference's."""
        eps = 1e-7 if torch.get_default_dtype() == torch.float32 else 1e-16
        if self.ntherm >= self.nstep:
            raise ValueError("Thermalisation longer than trajectory")
        with torch.no_grad():
            if self.ntherm < 0:
                self.ntherm = self.nstep + self.ntherm
            self.walkers.initialize(pos=pos)
            if self.logspace:
                def density(x):
                    return torch.log(pdf(x))
            else:
                density = pdf
            fx = density(self.walkers.pos)
            fx[fx == 0] = eps
            kept, naccept = [], 0
            tstart = time.time()
            for istep in range(self.nstep):
                for ielec in self.fixed_id_elec_list:
                    trial = self._trial_positions(ielec)
                    ftrial = density(trial)
                    if self.logspace:
                        ratio = ftrial - fx
                    else:
                        ftrial[ftrial == 0.0] = eps
                        ratio = ftrial / fx
                    take = self._accept_ratio(ratio)
                    naccept += int(take.sum())
                    self.walkers.pos[take, :] = trial[take, :]
                    fx[take] = ftrial[take]
                    fx[fx == 0] = eps
                if istep >= self.ntherm and (istep - self.ntherm) % self.ndecor == 0:
                    kept.append(self.walkers.pos.to("cpu").clone())
            self.last_acceptance = naccept / max(
                1, self.walkers.nwalkers * self._move_per_iter * self.nstep)
            if with_tqdm:
                dt = time.time() - tstart
                log.info("   Acceptance rate     : %1.2f %%", self.last_acceptance * 100)
                log.info("   Timing statistics   : %1.2f steps/sec.", self.nstep / dt)
        return self.symmetry(torch.cat(kept)).requires_grad_()

    def _trial_positions(self, ielec):
        """Trial walkers: every electron displaced (all-elec, or one electron
        in total), else one electron per walker, ``ielec`` or a random one
        (metropolis.py:227-254)."""
        nw = self.walkers.nwalkers
        if self.nelec == 1 or self.movedict["type"] == "all-elec":
            return self.walkers.pos + self._displacement(self.nelec)
        trial = self.walkers.pos.clone().view(nw, self.nelec, self.ndim)
        if ielec is None:
            which = torch.LongTensor(nw).random_(0, self.nelec)
        else:
            which = torch.LongTensor(nw).fill_(ielec)
        trial[range(nw), which, :] += self._displacement(1)
        return trial.view(nw, self.nelec * self.ndim)

    def _displacement(self, nmoved):
        """(nwalkers, 3 nmoved) displacements: uniform in [-step, step] or the
        normal law of ``configure_move`` (metropolis.py:256-277)."""
        nw = self.walkers.nwalkers
        if self._normal is None:
            u = torch.rand((nw, nmoved, self.ndim), device=self.device)
            return self.step_size * (2.0 * u.view(nw, nmoved * self.ndim) - 1.0)
        d = self._normal.sample((nw, nmoved)).to(self.device)
        return d.view(nw, nmoved * self.ndim)

    def _accept_ratio(self, ratio):
        """min(1, r) - u >= 0, or min(0, log r) - log u >= 0 with logspace
        (metropolis.py:279-298); u drawn like the ratio."""
        if self.logspace:
            ratio[ratio > 0] = 0.0
            tau = torch.log(torch.rand_like(ratio))
        else:
            ratio[ratio > 1] = 1.0
            tau = torch.rand_like(ratio)
        return (ratio - tau >= 0).reshape(-1).type(torch.bool)
