"""Slater-Jastrow wave function (drop-in for
``qmctorch.wavefunction.SlaterJastrow`` and its base ``WaveFunction``,
``qmctorch/wavefunction/slater_jastrow.py:30-482``, ``wf_base.py:7-277``).

``forward`` / ``pdf`` / ``local_energy`` / ``kinetic_energy`` run the fused
one-thread-per-walker kernels (``qmc_wf_psi``, ``qmc_wf_local_energy``); the
submodules ``ao, mo, jastrow, pool, fc`` keep the reference's call signatures
and run the staged kernels. State-dict names match the reference
(``ao.bas_exp``, ``ao.atom_coords``, ``mo.mo_modifier``,
``jastrow.jastrow_kernel.weight``, ``fc.weight``; with a list of Jastrow factors
``jastrow.jastrow_terms.<k>.jastrow_kernel.weight``).
"""
from __future__ import annotations

import logging

import torch
from torch import nn

from .. import _lib
from . import runtime as rt
from .jastrows import CombineJastrow, JastrowFactorElectronElectron, PadeJastrowKernel
from .orbitals import AtomicOrbitals, MolecularOrbitals
from .pooling import SlaterPooling
from .tables import OrbitalConfigurations

log = logging.getLogger("qmctorch_gb300")


class WaveFunction(nn.Module):
    """Base class (wf_base.py:7-277)."""

    def __init__(self, nelec, ndim, kinetic="auto", cuda=False):
        super().__init__()
        self.ndim = ndim
        self.nelec = nelec
        self.ndim_tot = nelec * ndim
        self.kinetic = kinetic
        self.cuda = cuda
        self.device = torch.device("cuda") if cuda else torch.device("cpu")

    def energy(self, pos):
        return torch.mean(self.local_energy(pos))

    def variance(self, pos):
        return torch.var(self.local_energy(pos))

    def sampling_error(self, eloc):
        return torch.sqrt(eloc.var() / eloc.shape[0])

    def _energy_variance(self, pos):
        el = self.local_energy(pos)
        return torch.mean(el), torch.var(el)

    def _energy_variance_error(self, pos):
        el = self.local_energy(pos)
        return torch.mean(el), torch.var(el), self.sampling_error(el)

    def get_number_parameters(self):
        return sum(p.numel() for p in self.parameters() if p.requires_grad)

    def load(self, filename, group="wf_opt", model="best"):
        """Load a state dict saved with ``torch.save`` (HDF5 is not available)."""
        data = torch.load(filename)
        if isinstance(data, dict) and "model_state_dict" in data:
            data = data["model_state_dict"]
        self.load_state_dict(data)


PRECISIONS = {"fp64": 0, "mixed": 1}


class _PsiFunction(torch.autograd.Function):
    """psi with a hand-written adjoint (``qmc_wf_psi_adjoint``) for the
    trainable parameters; AO values are recomputed in the backward pass.
    Gradients with respect to the electron positions are not provided."""

    @staticmethod
    def forward(ctx, x, bas_exp, mo_modifier, jastrow_w, jastrow_en_w, fc_weight, wf):
        ctx.wf = wf
        xd = rt.dev64(x, rt.cuda_device()).reshape(-1, wf.ndim_tot)
        ctx.save_for_backward(xd)
        return wf._psi(xd).reshape(-1, 1).to(device=x.device, dtype=x.dtype)

    @staticmethod
    def backward(ctx, gout):
        (xd,) = ctx.saved_tensors
        grads = ctx.wf._psi_adjoint(xd, gout.reshape(-1))
        need = ctx.needs_input_grad
        return (None,) + tuple(g if need[i + 1] else None for i, g in enumerate(grads)) + (None,)


class _ElocFunction(torch.autograd.Function):
    """Local energy with a hand-written adjoint (``qmc_wf_local_energy_adjoint``)
    for the trainable parameters, positions held fixed; AO values and
    derivatives are recomputed in the backward pass."""

    @staticmethod
    def forward(ctx, x, bas_exp, mo_modifier, jastrow_w, jastrow_en_w, fc_weight, wf):
        ctx.wf = wf
        xd = rt.dev64(x, rt.cuda_device()).reshape(-1, wf.ndim_tot)
        ctx.save_for_backward(xd)
        el, _ = wf._eloc(xd)
        return el.reshape(-1, 1).to(device=x.device, dtype=x.dtype)

    @staticmethod
    def backward(ctx, gout):
        (xd,) = ctx.saved_tensors
        grads = ctx.wf._adjoint(xd, gout.reshape(-1), "qmc_wf_local_energy_adjoint",
                                "qmc_eloc_adjoint_scratch_bytes")
        need = ctx.needs_input_grad
        return (None,) + tuple(g if need[i + 1] else None for i, g in enumerate(grads)) + (None,)


class SlaterJastrow(WaveFunction):
    """``precision`` (keyword added to the reference signature) selects the
    arithmetic of the fused psi / local-energy / Metropolis kernels: "fp64"
    (the plain method) or "mixed" (FP32 AO, AO->MO, Jastrow and Slater LU;
    FP64 determinant products, sums and one refinement step of the solves
    feeding the kinetic energy). Default: "fp64" when torch's default dtype is
    float64, else "mixed" (the reference's single-precision switch)."""

    def __init__(self, mol, jastrow="default", backflow=None, configs="ground_state",
                 kinetic="jacobi", cuda=False, include_all_mo=True, mix_mo=False,
                 orthogonalize_mo=False, precision=None):
        super().__init__(mol.nelec, 3, kinetic, cuda)
        if precision is None:
            precision = "fp64" if torch.get_default_dtype() == torch.float64 else "mixed"
        if precision not in PRECISIONS:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        if backflow is not None:
            raise NotImplementedError("backflow orbitals are not on the GB300 path")
        if not include_all_mo and isinstance(configs, str) and configs.startswith("cas("):
            raise ValueError("CAS calculation only possible with include_all_mo=True")
        self.mol = mol
        self.atoms = mol.atoms
        self.natom = mol.natom
        # configurations (slater_jastrow.py:158-169)
        self.orb_confs = OrbitalConfigurations(mol)
        self.configs_method = configs if isinstance(configs, str) else "explicit"
        self.configs = self.orb_confs.get_configs(configs)
        self.nci = len(self.configs[0])
        self.highest_occ_mo = int(max(self.configs[0].max(), self.configs[1].max())) + 1
        # layers
        self.use_backflow = False
        self.ao = AtomicOrbitals(mol, False)
        self.include_all_mo = include_all_mo
        self.nmo_opt = mol.basis.nmo if include_all_mo else self.highest_occ_mo
        self.mo = MolecularOrbitals(mol, include_all_mo, self.highest_occ_mo, mix_mo,
                                    orthogonalize_mo, False)
        self.mo.precision = precision
        self.pool = SlaterPooling(self.configs_method, self.configs, mol, False)
        self.fc = nn.Linear(self.nci, 1, bias=False)
        self.fc.weight.data.fill_(0.0)
        self.fc.weight.data[0][0] = 1.0
        if jastrow is None:
            self.jastrow = None
            self.use_jastrow = False
        else:
            self.use_jastrow = True
            if isinstance(jastrow, str) and jastrow == "default":
                self.jastrow = JastrowFactorElectronElectron(mol, PadeJastrowKernel)
            elif isinstance(jastrow, list):
                self.jastrow = CombineJastrow(jastrow)
            elif isinstance(jastrow, nn.Module):
                self.jastrow = jastrow
            else:
                raise TypeError("Jastrow factor not supported.")
            rt.jastrow_parts(self.jastrow)  # the kernels' factors: Pade e-e and / or e-n
            self.jastrow_type = repr(self.jastrow)
        jastrow_modules = [self.jastrow] if self.jastrow is not None else []
        if isinstance(self.jastrow, CombineJastrow):
            jastrow_modules += list(self.jastrow.jastrow_terms)
        for m in [self.mo, self.pool] + jastrow_modules:
            object.__setattr__(m, "_ao_module", self.ao)
        # kinetic energy: the Jacobi trace formula; "auto" (autograd in the
        # reference, wf_base.py:142-182) evaluates the same quantity
        self.kinetic_method = kinetic
        self.gradients = self.gradients_jacobi
        self.kinetic_energy = self.kinetic_energy_jacobi
        self._enuc_cache = (None, 0.0)
        self._desc_memo = rt.DescMemo()
        self._no_jastrow_w = torch.zeros(1)
        if cuda:
            self.device = rt.cuda_device()
            self.to(self.device)

    # -- descriptors ----------------------------------------------------------
    def nuclear_repulsion(self):
        """V_nn (wf_base.py:97-116)."""
        c = self.ao.atom_coords.detach().to("cpu", torch.float64)
        if self._enuc_cache[0] is None or not torch.equal(self._enuc_cache[0], c):
            z = self.ao.atomic_number
            v = 0.0
            for a in range(self.natom - 1):
                for b in range(a + 1, self.natom):
                    v += z[a] * z[b] / float(torch.sqrt(((c[a] - c[b]) ** 2).sum()))
            self._enuc_cache = (c, v)
        return self._enuc_cache[1]

    def _desc(self, device):
        """The kernels' descriptor of this wave function on ``device``: the
        last one built while its parameters keep the values it was built from
        (``rt.DescMemo``), else a new one."""
        jastrow = self.jastrow if self.use_jastrow else None
        key = (str(device), self.precision, self.highest_occ_mo, self.mol.nup, self.mol.ndown,
               id(self.ao), id(self.mo), id(self.pool), id(jastrow), id(self.fc))
        src = rt.desc_sources(self.ao, mo=self.mo, jastrow=jastrow, fc=self.fc)
        memo = self.__dict__.get("_desc_memo")
        if memo is None:
            memo = self._desc_memo = rt.DescMemo()
        call = memo.get(key, src, device)
        if call is not None:
            return call
        call = rt.build_desc(device, self.ao, mo=self.mo, pool=self.pool, jastrow=jastrow,
                             fc=self.fc, nup=self.mol.nup, ndown=self.mol.ndown,
                             nmo_used=self.highest_occ_mo, e_nuc=self.nuclear_repulsion(),
                             precision=PRECISIONS[self.precision])
        return memo.put(key, src, device, call)

    # -- fused evaluations ----------------------------------------------------
    def _psi(self, pos):
        device = rt.cuda_device()
        x = rt.dev64(pos, device).reshape(-1, self.ndim_tot)
        nb = x.shape[0]
        call = self._desc(device)
        lib = _lib.lib()
        scr = rt.scratch(lib.qmc_scratch_bytes(call.ref, nb, 0), device)
        psi = torch.empty(nb, dtype=rt.F64, device=device)
        _lib.check(lib.qmc_wf_psi(call.ref, rt.ptr(x), nb, rt.ptr(psi), rt.ptr(scr), scr.numel(),
                                  rt.stream_handle()), "qmc_wf_psi")
        return psi

    def _eloc(self, pos, want_kin=False):
        device = rt.cuda_device()
        x = rt.dev64(pos, device).reshape(-1, self.ndim_tot)
        nb = x.shape[0]
        call = self._desc(device)
        lib = _lib.lib()
        scr = rt.scratch(lib.qmc_scratch_bytes(call.ref, nb, 1), device)
        el = torch.empty(nb, dtype=rt.F64, device=device)
        kin = torch.empty(nb, dtype=rt.F64, device=device) if want_kin else None
        _lib.check(lib.qmc_wf_local_energy(call.ref, rt.ptr(x), nb, rt.ptr(el), rt.ptr(kin), None,
                                           rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   "qmc_wf_local_energy")
        return el, kin

    def forward(self, x, ao=None):
        """psi = J * sum_n c_n D_up D_down -> (nbatch, 1) (slater_jastrow.py:243-286).
        Differentiable with respect to ao.bas_exp, mo.mo_modifier,
        jastrow.jastrow_kernel.weight and fc.weight (hand-written adjoint)."""
        if ao is not None:
            out = self.fc(self.pool(self.mo(ao)))
            if self.use_jastrow:
                out = self.jastrow(x) * out
            return out
        params = self._trainable()
        if torch.is_grad_enabled() and any(p.requires_grad for p in params):
            return _PsiFunction.apply(x, *params, self)
        return self._psi(x).reshape(-1, 1).to(device=x.device, dtype=x.dtype)

    def _psi_adjoint(self, x, gout):
        """Parameter gradients of sum_w gout[w] psi_w (qmc_wf_psi_adjoint)."""
        return self._adjoint(x, gout, "qmc_wf_psi_adjoint", "qmc_adjoint_scratch_bytes")

    def _adjoint(self, x, gout, fn, scratch_fn):
        """Parameter gradients of sum_w gout[w] f_w by the adjoint entry point
        ``fn`` (psi or the local energy)."""
        device = rt.cuda_device()
        nb = x.shape[0]
        call = self._desc(device)
        bt = self.ao.device_tables(device)
        nmu = self.highest_occ_mo
        lib = _lib.lib()
        g = rt.dev64(gout, device)
        g_exp = torch.zeros(bt.nentries, dtype=rt.F64, device=device)
        g_W = torch.zeros((self.ao.norb, nmu), dtype=rt.F64, device=device)
        g_w = torch.zeros(2, dtype=rt.F64, device=device)  # e-e and e-n Pade weights
        g_ci = torch.zeros(self.nci, dtype=rt.F64, device=device)
        scr = rt.scratch(getattr(lib, scratch_fn)(call.ref, nb), device)
        _lib.check(getattr(lib, fn)(call.ref, rt.ptr(x), nb, rt.ptr(g), rt.ptr(bt.t["w_entry"]),
                                    bt.nentries, rt.ptr(g_exp), rt.ptr(g_W), nmu, rt.ptr(g_w),
                                    rt.ptr(g_ci), rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   fn)
        mod = self.mo.mo_modifier
        g_mod = torch.zeros(mod.shape, dtype=rt.F64, device=device)
        g_mod[:, :nmu] = g_W * rt.dev64(self.mo.mo_scf, device)[:, :nmu]
        cast = lambda t, p: t.to(device=p.device, dtype=p.dtype).reshape(p.shape)  # noqa: E731
        jw, jwn = self._jastrow_weights()
        return (cast(g_exp, self.ao.bas_exp), cast(g_mod, mod), cast(g_w[:1], jw),
                cast(g_w[1:], jwn), cast(g_ci, self.fc.weight))

    def _jastrow_weights(self):
        """(e-e Pade weight, e-n Pade weight) parameters, a fixed placeholder for
        an absent factor."""
        ee, en = rt.jastrow_parts(self.jastrow if self.use_jastrow else None)
        return (ee.jastrow_kernel.weight if ee is not None else self._no_jastrow_w,
                en.jastrow_kernel.weight if en is not None else self._no_jastrow_w)

    def _trainable(self):
        """The parameters the hand-written adjoints differentiate."""
        jw, jwn = self._jastrow_weights()
        return (self.ao.bas_exp, self.mo.mo_modifier, jw, jwn, self.fc.weight)

    def pdf(self, pos, return_grad=False):
        """psi^2 -> (nbatch,) (wf_base.py:241-247)."""
        if return_grad:
            return self.gradients(pos, pdf=True)
        psi = self._psi(pos)
        return (psi * psi).to(device=pos.device, dtype=pos.dtype)

    def local_energy(self, pos):
        """E_L = KE + V_en + V_ee + V_nn -> (nbatch, 1) (wf_base.py:184-215).
        Differentiable with respect to ao.bas_exp, mo.mo_modifier,
        jastrow.jastrow_kernel.weight and fc.weight (hand-written adjoint)."""
        params = self._trainable()
        if torch.is_grad_enabled() and any(p.requires_grad for p in params):
            return _ElocFunction.apply(pos, *params, self)
        el, _ = self._eloc(pos)
        return el.reshape(-1, 1).to(device=pos.device, dtype=pos.dtype)

    def kinetic_energy_jacobi(self, x, **kwargs):
        """-1/2 lap(psi)/psi by the Jacobi trace formula (slater_jastrow.py:312-344)."""
        el, kin = self._eloc(x, want_kin=True)
        return kin.reshape(-1, 1).to(device=x.device, dtype=x.dtype)

    kinetic_energy_autograd = kinetic_energy_jacobi

    def gradients_jacobi(self, x, sum_grad=False, pdf=False):
        """d psi / d r (or d psi^2 / d r with pdf=True) -> (nbatch, 3*nelec), by
        the Jacobi formula (slater_jastrow.py:346-447); FP64. ``sum_grad`` is
        accepted and, as in the reference, not used."""
        device = rt.cuda_device()
        xd = rt.dev64(x, device).reshape(-1, self.ndim_tot)
        nb = xd.shape[0]
        call = self._desc(device)
        lib = _lib.lib()
        scr = rt.scratch(lib.qmc_grad_scratch_bytes(call.ref, nb), device)
        out = torch.empty((nb, self.ndim_tot), dtype=rt.F64, device=device)
        _lib.check(lib.qmc_wf_gradients(call.ref, rt.ptr(xd), nb, 1 if pdf else 0, rt.ptr(out),
                                        rt.ptr(scr), scr.numel(), rt.stream_handle()),
                   "qmc_wf_gradients")
        return out.to(device=x.device, dtype=x.dtype)

    gradients_autograd = gradients_jacobi

    def _potentials(self, pos, en=True, ee=True):
        device = rt.cuda_device()
        x = rt.dev64(pos, device).reshape(-1, self.ndim_tot)
        nb = x.shape[0]
        call = self._desc(device)
        ven = torch.empty(nb, dtype=rt.F64, device=device) if en else None
        vee = torch.empty(nb, dtype=rt.F64, device=device) if ee else None
        _lib.check(_lib.lib().qmc_potentials(call.ref, rt.ptr(x), nb, rt.ptr(ven), rt.ptr(vee),
                                             rt.stream_handle()), "qmc_potentials")
        return ven, vee

    def nuclear_potential(self, pos):
        """V_en (wf_base.py:72-95) -> (nbatch, 1)."""
        v, _ = self._potentials(pos, ee=False)
        return v.reshape(-1, 1).to(device=pos.device, dtype=pos.dtype)

    def electronic_potential(self, pos):
        """V_ee (wf_base.py:49-70) -> (nbatch, 1)."""
        _, v = self._potentials(pos, en=False)
        return v.reshape(-1, 1).to(device=pos.device, dtype=pos.dtype)

    # -- staged helpers (slater_jastrow.py:288-310) ------------------------------
    def ao2mo(self, ao):
        return self.mo(ao)

    def pos2mo(self, x, derivative=0, sum_grad=True):
        return self.ao2mo(self.ao(x, derivative=derivative, sum_grad=sum_grad))

    def log_data(self):
        log.info("  Wave Function")
        log.info("  Jastrow factor      : %s", self.use_jastrow)
        log.info("  Highest MO included : %d", self.nmo_opt)
        log.info("  Configurations      : %s", self.configs_method)
        log.info("  Number of confs     : %d", self.nci)
        log.info("  Kinetic energy      : %s", self.kinetic_method)
        log.info("  Number var  param   : %d", self.get_number_parameters())
        log.info("  Cuda support        : %s", self.cuda)
