"""Slater determinant pooling (drop-in for
``qmctorch.wavefunction.pooling.slater_pooling.SlaterPooling``).

Determinants and trace operators are computed by ``qmc_slater`` with the
recipes of :class:`tables.ConfigTables`: excitation mode for
``ground_state`` / ``single(n,m)`` / ``single_double(n,m)`` (the reference's
``det_single_double`` / ``operator_single_double``), explicit mode for
``cas(n,m)`` and user tuples (``det_explicit`` / ``operator_explicit``).
"""
from __future__ import annotations

import operator as _operator

import torch
from torch import nn

from .. import _lib
from . import runtime as rt
from .tables import ConfigTables, get_unique_excitation


class SlaterPooling(nn.Module):
    def __init__(self, config_method, configs, mol, cuda=False):
        super().__init__()
        self.config_method = config_method
        self.configs = configs
        self.nconfs = len(configs[0])
        self.index_max_orb_up = int(configs[0].max()) + 1
        self.index_max_orb_down = int(configs[1].max()) + 1
        self.unique_excitation, self.index_unique_excitation = get_unique_excitation(configs)
        self.nmo = mol.basis.nmo
        self.nup = mol.nup
        self.ndown = mol.ndown
        self.nelec = self.nup + self.ndown
        self.use_explicit_operator = False
        self._tables = ConfigTables(config_method, configs, self.nup, self.ndown)
        self._tables_device = None
        object.__setattr__(self, "_ao_module", None)  # set by the owning wave function
        self._mol = mol

    def device_tables(self, device):
        if self._tables_device != device:
            self._tables.to(device)
            self._tables_device = device
        return self._tables

    def _call(self, mo, bop):
        device = rt.cuda_device()
        if self._ao_module is None:
            from .orbitals import AtomicOrbitals
            object.__setattr__(self, "_ao_module", AtomicOrbitals(self._mol))
        m = rt.dev64(mo, device)
        nb, ne, ld = m.shape
        b = rt.dev64(bop, device) if bop is not None else None
        nmu = max(self._tables.max_orb)
        call = rt.build_desc(device, self._ao_module, pool=self, nup=self.nup, ndown=self.ndown,
                             nmo_used=nmu)
        call.desc.nmo = ld
        # ci weights are not read by qmc_slater; use ones
        lib = _lib.lib()
        scr = rt.scratch(lib.qmc_scratch_bytes(call.ref, nb, 1), device)
        dets = torch.empty((nb, self.nconfs), dtype=rt.F64, device=device)
        opv = torch.empty((nb, self.nconfs), dtype=rt.F64, device=device) if b is not None else None
        _lib.check(lib.qmc_slater(call.ref, rt.ptr(m), rt.ptr(b), ld, nb, rt.ptr(dets),
                                  rt.ptr(opv), rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   "qmc_slater")
        return dets, opv

    def forward(self, input):
        """Determinants of the configurations (slater_pooling.py:64-80)."""
        dets, _ = self._call(input, None)
        return dets.to(device=input.device, dtype=input.dtype)

    def operator(self, mo, bop, op=_operator.add, op_squared=False, inv_mo=None):
        """Tr(A^-1 B) per configuration, up and down spins added
        (slater_pooling.py:262-306)."""
        if op_squared:
            raise NotImplementedError("squared operators are not on the GB300 path")
        if op is not _operator.add:
            raise NotImplementedError("only the summed (op.add) spin combination is provided")
        if bop.ndim == 4:
            outs = [self._call(mo, bop[i])[1] for i in range(bop.shape[0])]
            return torch.stack(outs, 0).to(device=mo.device, dtype=mo.dtype)
        return self._call(mo, bop)[1].to(device=mo.device, dtype=mo.dtype)
