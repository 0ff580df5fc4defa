"""Electron-nucleus Pade-Jastrow factor (drop-ins for
``JastrowFactorElectronNuclei`` and its ``PadeJastrowKernel``,
``qmctorch/wavefunction/jastrows/elec_nuclei/``).

J = exp(sum_{i,A} r_iA / (1 + w r_iA)): the same static weight 1 for every
electron-nucleus pair (pade_jastrow_kernel.py:8-46). The parameter keeps the
reference name ``jastrow_kernel.weight``. Values come from ``qmc_jastrow_en``;
inside a wave function the term is fused into the psi, local-energy,
Metropolis, gradient and adjoint kernels.
"""
from __future__ import annotations

import torch
from torch import nn

from ... import _lib
from .. import runtime as rt


class PadeJastrowKernel(nn.Module):
    """B_iA = r_iA / (1 + w r_iA) (elec_nuclei/kernels/pade_jastrow_kernel.py:8-46)."""

    def __init__(self, nup, ndown, atomic_pos, cuda, w=1.0):
        super().__init__()
        self.nup, self.ndown = nup, ndown
        self.nelec = nup + ndown
        self.atoms = atomic_pos
        self.natoms = atomic_pos.shape[0]
        self.ndim = 3
        self.cuda = cuda
        self.weight = nn.Parameter(torch.as_tensor([w]), requires_grad=True)
        self.static_weight = torch.as_tensor([1.0])
        self.requires_autograd = True

    def forward(self, r):
        """Kernel values for a tensor of electron-nucleus distances."""
        return self.static_weight.to(r) * r / (1.0 + self.weight.to(r) * r)


class JastrowFactorElectronNuclei(nn.Module):
    """J = prod_{i,A} exp(B(r_iA)) with gradients and laplacians
    (jastrow_factor_electron_nuclei.py:9-161)."""

    def __init__(self, mol, jastrow_kernel=PadeJastrowKernel, kernel_kwargs={}, cuda=False):
        super().__init__()
        if jastrow_kernel is not PadeJastrowKernel:
            raise NotImplementedError("the GB300 kernels implement the Pade e-n kernel")
        self.nup, self.ndown = mol.nup, mol.ndown
        self.nelec = mol.nup + mol.ndown
        self.cuda = cuda
        atomic_pos = torch.as_tensor(mol.atom_coords)
        self.atoms = atomic_pos
        self.natoms = atomic_pos.shape[0]
        self.ndim = 3
        self.jastrow_kernel = jastrow_kernel(mol.nup, mol.ndown, atomic_pos, cuda,
                                             **kernel_kwargs)
        self.requires_autograd = self.jastrow_kernel.requires_autograd
        object.__setattr__(self, "_ao_module", None)  # set by the owning wave function
        self._mol = mol

    def __repr__(self):
        return "en -> " + self.jastrow_kernel.__class__.__name__

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
        _lib.check(_lib.lib().qmc_jastrow_en(call.ref, rt.ptr(x), nb, rt.ptr(jast), rt.ptr(dj),
                                             rt.ptr(d2j), int(bool(sum_grad)), rt.stream_handle()),
                   "qmc_jastrow_en")
        back = lambda t: t.to(device=pos.device, dtype=pos.dtype)  # noqa: E731
        if derivative == 0:
            return back(jast)
        if derivative == 1:
            return back(dj)
        if derivative == 2:
            return back(d2j)
        return back(jast), back(dj), back(d2j)


JastrowFactor = JastrowFactorElectronNuclei  # name exported by qmctorch.wavefunction.jastrows.elec_nuclei
