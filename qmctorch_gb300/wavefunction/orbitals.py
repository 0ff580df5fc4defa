"""Atomic and molecular orbital layers (drop-ins for
``qmctorch.wavefunction.orbitals.atomic_orbitals.AtomicOrbitals`` and
``qmctorch.wavefunction.orbitals.molecular_orbitals.MolecularOrbitals``).

Parameters and state-dict names follow the reference: ``ao.bas_exp``,
``ao.atom_coords`` (atomic_orbitals.py:33-36, 55-56) and ``mo.mo_modifier``
(molecular_orbitals.py:42-45). The values are computed by ``qmc_ao_eval`` /
``qmc_mo_eval``.
"""
from __future__ import annotations

import numpy as np
import torch
from torch import nn

from .. import _lib
from . import runtime as rt
from .tables import BasisTables, entry_norms


class AtomicOrbitals(nn.Module):
    """AO values, gradients and laplacians of cartesian Gaussian (pyscf
    layout) or Slater-type (ADF layout: r^kr exp(-a r), or exp(-a r) for
    radial_type "sto_pure") orbitals (atomic_orbitals.py:15-218)."""

    def __init__(self, mol, cuda=False):
        super().__init__()
        dtype = torch.get_default_dtype()
        self.nelec = mol.nelec
        self.norb = int(mol.basis.nao)
        self.ndim = 3
        self.atom_coords = nn.Parameter(
            torch.as_tensor(np.asarray(mol.basis.atom_coords_internal)).type(dtype))
        self.atom_coords.requires_grad = True
        self.natoms = len(self.atom_coords)
        self.atomic_number = mol.atomic_number
        self.nshells = torch.as_tensor(np.asarray(mol.basis.nshells))
        self.index_ctr = torch.as_tensor(np.asarray(mol.basis.index_ctr))
        self.nctr_per_ao = torch.as_tensor(np.asarray(mol.basis.nctr_per_ao))
        self.contract = not len(torch.unique(self.index_ctr)) == len(self.index_ctr)
        self.bas_coeffs = torch.as_tensor(np.asarray(mol.basis.bas_coeffs)).type(dtype)
        self.bas_exp = nn.Parameter(torch.as_tensor(np.asarray(mol.basis.bas_exp)).type(dtype))
        self.bas_exp.requires_grad = True
        self.harmonics_type = mol.basis.harmonics_type
        self.radial_type = mol.basis.radial_type
        self.norm_cst = torch.as_tensor(entry_norms(mol.basis)).type(dtype)
        self._basis = mol.basis
        self._tables = BasisTables(mol.basis, np.asarray(mol.basis.bas_exp, dtype=np.float64))
        self._tables_version = None
        self._tables_device = None
        self._charge = {}
        self.backflow_trans = None
        self.cuda = cuda
        self.device = torch.device("cpu")
        if cuda:
            self.device = rt.cuda_device()
            self.to(self.device)

    def __repr__(self):
        return "AtomicOrbitals(%s, %s, %d -> (%d,%d) )" % (
            self.radial_type, self.harmonics_type, self.nelec * self.ndim, self.nelec, self.norb)

    # -- device tables ------------------------------------------------------
    def device_tables(self, device):
        """AO group tables on ``device``; regrouped if training made the
        exponents of one group diverge."""
        version = (self.bas_exp._version, self.bas_exp.data_ptr())
        if version != self._tables_version:
            values = self.bas_exp.detach().to("cpu", torch.float64).numpy()
            if not self._tables.still_valid(values):
                self._tables = BasisTables(self._basis, values)
                self._tables_device = None
            self._tables_version = version
        if self._tables_device != device:
            self._tables.to(device)
            self._tables_device = device
        return self._tables

    def atomic_charge(self, device):
        key = str(device)
        if key not in self._charge:
            self._charge[key] = torch.as_tensor(np.asarray(self.atomic_number, dtype=np.float64),
                                                device=device)
        return self._charge[key]

    # -- forward ------------------------------------------------------------
    def forward(self, pos, derivative=[0], sum_grad=True, sum_hess=True, one_elec=False):
        if not isinstance(derivative, list):
            derivative = [derivative]
        if not sum_grad:
            assert 1 in derivative
        if not sum_hess:
            assert 2 in derivative
        if derivative == [0]:
            mode = 0
        elif derivative == [1]:
            mode = 3 if sum_grad else 1
        elif derivative == [2]:
            if not sum_hess:
                raise NotImplementedError("per-axis AO second derivatives are not on the GB300 path")
            mode = 2
        elif derivative == [0, 1, 2]:
            mode = 4
        elif derivative == [3]:
            raise NotImplementedError("mixed AO second derivatives are not on the GB300 path")
        else:
            raise ValueError("derivative must be 0, 1, 2, 3 or [0, 1, 2, 3], got ", derivative)
        device = rt.cuda_device()
        nelec = 1 if one_elec else self.nelec
        x = rt.dev64(pos, device).reshape(-1, 3 * nelec)
        nb = x.shape[0]
        call = rt.build_desc(device, self, nelec=nelec)
        shape = (nb, nelec, self.norb)
        ao = torch.empty(shape, dtype=rt.F64, device=device) if mode in (0, 3, 4) else None
        dao = torch.empty(shape + (3,), dtype=rt.F64, device=device) if mode in (1, 4) else None
        d2ao = torch.empty(shape, dtype=rt.F64, device=device) if mode in (2, 4) else None
        _lib.check(_lib.lib().qmc_ao_eval(call.ref, rt.ptr(x), nb, mode, rt.ptr(ao), rt.ptr(dao),
                                          rt.ptr(d2ao), rt.stream_handle()), "qmc_ao_eval")
        back = lambda t: t.to(device=pos.device, dtype=pos.dtype)  # noqa: E731
        if mode == 4:
            return back(ao), back(dao), back(d2ao)
        return back({0: ao, 3: ao, 1: dao, 2: d2ao}[mode])

    def update(self, ao, pos, idelec):
        """AO matrix with one electron moved (atomic_orbitals.py:671-695)."""
        ao_new = ao.clone()
        ids, ide = idelec * 3, (idelec + 1) * 3
        ao_new[:, idelec, :] = self.forward(pos[:, ids:ide], one_elec=True).squeeze(1)
        return ao_new


class MolecularOrbitals(nn.Module):
    """MO = AO @ (mo_scf * mo_modifier) (molecular_orbitals.py:7-95).

    ``precision`` (set by the owning wave function; default from torch's
    default dtype as there) picks the kernel: "fp64" runs ``qmc_mo_eval``
    (FP64, exact to rounding), "mixed" runs ``qmc_mo_eval_tc`` (tensor cores,
    split-BF16 x3 with FP32 accumulation, error about 2e-5 of |AO| @ |W|)."""

    def __init__(self, mol, include_all_mo, highest_occ_mo, mix_mo, orthogonalize_mo, cuda):
        super().__init__()
        dtype = torch.get_default_dtype()
        self.precision = "fp64" if dtype == torch.float64 else "mixed"
        self.mol = mol
        self.mix_mo = mix_mo
        self.orthogonalize_mo = orthogonalize_mo
        if mix_mo:
            raise NotImplementedError("mix_mo is not supported")
        if orthogonalize_mo:
            raise Warning("orthogonalize_mo=True has no effect as mix_mo=False")
        self.include_all_mo = include_all_mo
        self.highest_occ_mo = highest_occ_mo
        self.nmo_opt = mol.basis.nmo if include_all_mo else highest_occ_mo
        mos = torch.as_tensor(np.asarray(mol.basis.mos)).type(dtype)
        if not include_all_mo:
            mos = mos[:, :highest_occ_mo]
        self.mo_scf = mos.contiguous().requires_grad_(False)
        self.mo_modifier = nn.Parameter(torch.ones_like(self.mo_scf, requires_grad=True)).type(dtype)
        self.mo_mixer = None
        object.__setattr__(self, "_ao_module", None)  # set by the owning wave function
        self.cuda = cuda
        self.device = torch.device("cpu")
        if cuda:
            self.device = rt.cuda_device()
            self.mo_scf = self.mo_scf.to(self.device)

    def _apply(self, fn, *args, **kwargs):
        out = super()._apply(fn, *args, **kwargs)
        self.mo_scf = fn(self.mo_scf)
        return out

    def forward(self, ao):
        device = rt.cuda_device()
        nao = ao.shape[-1]
        x = rt.dev64(ao, device).reshape(-1, nao)
        if self._ao_module is None:
            object.__setattr__(self, "_ao_module", AtomicOrbitals(self.mol))
        call = rt.build_desc(device, self._ao_module, mo=self)
        out = torch.empty((x.shape[0], self.mo_scf.shape[1]), dtype=rt.F64, device=device)
        fn = "qmc_mo_eval_tc" if self.precision == "mixed" else "qmc_mo_eval"
        lib = _lib.lib()
        _lib.check(getattr(lib, fn)(call.ref, rt.ptr(x), x.shape[0], rt.ptr(out),
                                    rt.stream_handle()), fn)
        if fn == "qmc_mo_eval_tc":
            # the pipelined kernel reports a wait that ran out by a status word
            _lib.check(lib.qmc_mo_eval_tc_status(rt.stream_handle()), fn)
        return out.reshape(*ao.shape[:-1], -1).to(device=ao.device, dtype=ao.dtype)
