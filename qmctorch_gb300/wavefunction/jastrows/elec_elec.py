"""Electron-electron Pade-Jastrow factor (drop-ins for
``JastrowFactorElectronElectron`` and ``PadeJastrowKernel``,
``qmctorch/wavefunction/jastrows/elec_elec/``).

The parameter keeps the reference name ``jastrow.jastrow_kernel.weight``
(pade_jastrow_kernel.py:28). Values come from ``qmc_jastrow_ee``.
"""
from __future__ import annotations

import torch
from torch import nn

from ... import _lib
from .. import runtime as rt


class PadeJastrowKernel(nn.Module):
    """B_ij = w0 r_ij / (1 + w r_ij); w0 = 0.25 for same-spin pairs and 0.5 for
    opposite-spin pairs, as the reference code builds it
    (pade_jastrow_kernel.py:34-66)."""

    def __init__(self, nup, ndown, cuda, w=1.0):
        super().__init__()
        self.nup, self.ndown = nup, ndown
        self.cuda = cuda
        self.weight = nn.Parameter(torch.as_tensor([w]), requires_grad=True)
        self.requires_autograd = False

    def get_static_weight(self):
        n = self.nup + self.ndown
        sw = torch.full((n, n), 0.5)
        sw[: self.nup, : self.nup] = 0.25
        sw[self.nup:, self.nup:] = 0.25
        return sw.masked_select(torch.triu(torch.ones(n, n), diagonal=1).bool())


class JastrowFactorElectronElectron(nn.Module):
    """J = exp(sum_{i<j} B(r_ij)) with gradients and laplacians
    (jastrow_factor_electron_electron.py:11-260)."""

    def __init__(self, mol, jastrow_kernel=PadeJastrowKernel, kernel_kwargs={}, scale=False,
                 scale_factor=0.6, cuda=False):
        super().__init__()
        if jastrow_kernel is not PadeJastrowKernel:
            raise NotImplementedError("the GB300 Jastrow kernel implements the Pade e-e kernel")
        if scale:
            raise NotImplementedError("scaled e-e distances are not on the GB300 path")
        self.nup, self.ndown = mol.nup, mol.ndown
        self.nelec = mol.nup + mol.ndown
        self.ndim = 3
        self.cuda = cuda
        self.jastrow_kernel = jastrow_kernel(mol.nup, mol.ndown, cuda, **kernel_kwargs)
        self.requires_autograd = self.jastrow_kernel.requires_autograd
        object.__setattr__(self, "_ao_module", None)  # set by the owning wave function
        self._mol = mol

    def __repr__(self):
        return "ee -> " + self.jastrow_kernel.__class__.__name__

    def forward(self, pos, derivative=0, sum_grad=True):
        device = rt.cuda_device()
        assert pos.shape[1] == self.nelec * self.ndim
        if self._ao_module is None:
            from ..orbitals import AtomicOrbitals
            object.__setattr__(self, "_ao_module", AtomicOrbitals(self._mol))
        x = rt.dev64(pos, device)
        nb = x.shape[0]
        call = rt.build_desc(device, self._ao_module, jastrow=self, nup=self.nup,
                             ndown=self.ndown)
        want = [0, 1, 2] if derivative == [0, 1, 2] else [derivative]
        jast = torch.empty((nb, 1), dtype=rt.F64, device=device)
        dj = None
        if 1 in want:
            shape = (nb, self.nelec) if sum_grad else (nb, 3, self.nelec)
            dj = torch.empty(shape, dtype=rt.F64, device=device)
        d2j = torch.empty((nb, self.nelec), dtype=rt.F64, device=device) if 2 in want else None
        _lib.check(_lib.lib().qmc_jastrow_ee(call.ref, rt.ptr(x), nb, rt.ptr(jast), rt.ptr(dj),
                                             rt.ptr(d2j), int(bool(sum_grad)), rt.stream_handle()),
                   "qmc_jastrow_ee")
        back = lambda t: t.to(device=pos.device, dtype=pos.dtype)  # noqa: E731
        if derivative == 0:
            return back(jast)
        if derivative == 1:
            return back(dj)
        if derivative == 2:
            return back(d2j)
        return back(jast), back(dj), back(d2j)


JastrowFactor = JastrowFactorElectronElectron  # name exported by qmctorch.wavefunction.jastrows.elec_elec
