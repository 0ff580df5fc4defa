"""Call plumbing between the torch modules and ``libqmc_gb300``: device
placement, the ``qmc_wf_desc`` of each call and scratch buffers.

The kernels compute in FP64 on the current CUDA device. Inputs on another
device or dtype are copied for the call and outputs are returned on the
input's device and dtype, so the modules accept the CPU tensors the reference
API is usually called with.
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib

F64 = torch.float64


def cuda_device():
    if not torch.cuda.is_available():
        raise RuntimeError("qmctorch_gb300 runs its kernels on a CUDA GPU (sm_103a); "
                           "no CUDA device is visible")
    return torch.device("cuda", torch.cuda.current_device())


def dev64(t, device):
    """Contiguous FP64 copy of ``t`` on ``device`` (no copy if already there)."""
    t = t.detach() if isinstance(t, torch.Tensor) else torch.as_tensor(t)
    if t.device != device or t.dtype != F64 or not t.is_contiguous():
        t = t.to(device=device, dtype=F64).contiguous()
    return t


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


_DUMMY = {}


def dummies(device):
    key = str(device)
    if key not in _DUMMY:
        _DUMMY[key] = (torch.zeros(8, dtype=torch.int32, device=device),
                       torch.ones(8, dtype=F64, device=device))
    return _DUMMY[key]


def scratch(nbytes, device):
    return torch.empty(max(int(nbytes), 8), dtype=torch.uint8, device=device)


def walker_stats(eloc):
    """(mean, unbiased variance, sqrt(variance / n)) of the local energies by
    the compensated qmc_reduce_stats kernel; returned on eloc's device."""
    device = cuda_device()
    x = dev64(eloc.reshape(-1), device)
    n = x.numel()
    lib = _lib.lib()
    scr = scratch(lib.qmc_reduce_scratch_bytes(n), device)
    out = torch.empty(3, dtype=F64, device=device)
    _lib.check(lib.qmc_reduce_stats(ptr(x), n, ptr(out), ptr(scr), scr.numel(), stream_handle()),
               "qmc_reduce_stats")
    out = out.to(device=eloc.device, dtype=eloc.dtype)
    return out[0], out[1], out[2]


class Call:
    """A filled ``qmc_wf_desc`` plus the tensors its pointers refer to."""

    def __init__(self, desc, keep):
        self.desc = desc
        self.keep = keep
        self.ref = ctypes.byref(desc)


def jastrow_parts(jastrow):
    """(e-e Pade factor or None, e-n Pade factor or None) of a Jastrow module:
    one factor, or a CombineJastrow of at most one of each. Anything else
    raises NotImplementedError (the kernels implement these two factors)."""
    from .jastrows import CombineJastrow, JastrowFactorElectronElectron, JastrowFactorElectronNuclei
    if jastrow is None:
        return None, None
    terms = list(jastrow.jastrow_terms) if isinstance(jastrow, CombineJastrow) else [jastrow]
    ee = [t for t in terms if isinstance(t, JastrowFactorElectronElectron)]
    en = [t for t in terms if isinstance(t, JastrowFactorElectronNuclei)]
    if len(ee) + len(en) != len(terms) or len(ee) > 1 or len(en) > 1:
        raise NotImplementedError("the GB300 kernels implement the Pade e-e and e-n Jastrow "
                                  "factors, at most one of each")
    return (ee[0] if ee else None), (en[0] if en else None)


def desc_sources(ao, mo=None, jastrow=None, fc=None):
    """The tensors whose values ``build_desc`` copies into a descriptor or
    points it at, in a fixed order."""
    src = [ao.atom_coords, ao.bas_exp]
    if mo is not None:
        src += [mo.mo_scf, mo.mo_modifier]
    ee, en = jastrow_parts(jastrow)
    if ee is not None:
        src.append(ee.jastrow_kernel.weight)
    if en is not None:
        src += [en.jastrow_kernel.weight, en.atoms]
    if fc is not None:
        src.append(fc.weight)
    return src


class DescMemo:
    """The last descriptor built for a wave function and what it was built
    from, so that repeated calls with unchanged parameters make no
    host-to-device copies. A host tensor is compared by value with a snapshot
    taken at build time (a write through ``.data`` does not advance a tensor's
    version counter, so versions are not trusted); a device FP64 contiguous
    tensor is used in place by the descriptor, so its identity and storage
    address are compared; a descriptor built from any other source (a device
    tensor that needed a conversion) is never reused."""

    def __init__(self):
        self.key = None
        self.snap = None
        self.call = None

    def __deepcopy__(self, memo):
        return DescMemo()

    def __getstate__(self):
        return {"key": None, "snap": None, "call": None}

    @staticmethod
    def _snapshot(t, device):
        t = t.detach()
        if t.device.type == "cpu":
            return t.clone()
        if t.device == device and t.dtype == F64 and t.is_contiguous():
            return t.data_ptr()
        return None

    def get(self, key, sources, device):
        if self.call is None or key != self.key or len(sources) != len(self.snap):
            return None
        for t, (ref, s) in zip(sources, self.snap):
            if t is not ref:
                return None
            if isinstance(s, torch.Tensor):
                td = t.detach()
                if td.device.type != "cpu" or td.dtype != s.dtype or td.shape != s.shape or \
                        not torch.equal(td, s):
                    return None
            elif (t.device != device or t.dtype != F64 or not t.is_contiguous()
                  or t.data_ptr() != s):
                return None
        return self.call

    def put(self, key, sources, device, call):
        snap = [(t, self._snapshot(t, device)) for t in sources]
        if any(s is None for _, s in snap):
            self.key = self.snap = self.call = None
        else:
            self.key, self.snap, self.call = key, snap, call
        return call


def build_desc(device, ao, mo=None, pool=None, jastrow=None, fc=None, nelec=None, nup=None,
               ndown=None, nmo_used=None, e_nuc=0.0, precision=0):
    """Fill a ``qmc_wf_desc`` from the modules of a wave function. Any module
    may be absent (a standalone AO or Jastrow call); its fields then point to
    placeholders the called kernel does not read."""
    di, dd = dummies(device)
    keep = [di, dd]
    d = _lib.WfDesc()
    nelec = ao.nelec if nelec is None else nelec
    d.nelec = nelec
    d.nup = nelec if nup is None else nup
    d.ndown = 0 if ndown is None else ndown
    d.natom = ao.natoms
    d.nao = ao.norb
    bt = ao.device_tables(device)
    keep.append(bt)  # its index tensors are pointed at by the descriptor
    coords = dev64(ao.atom_coords, device)
    charge = ao.atomic_charge(device)
    bexp = dev64(ao.bas_exp, device)
    keep += [coords, charge, bexp]
    d.ngroup, d.ngprim, d.nweight = bt.ngroup, bt.ngprim, bt.nweight
    d.contract = int(bt.contract)
    d.atom_coords, d.atom_charge = ptr(coords), ptr(charge)
    t = bt.t
    d.group_atom, d.group_prim, d.group_ao = ptr(t["group_atom"]), ptr(t["group_prim"]), ptr(
        t["group_ao"])
    d.gprim_entry, d.bas_exp, d.ao_k = ptr(t["gprim_entry"]), ptr(bexp), ptr(t["ao_k"])
    d.ao_wofs, d.ao_wd = ptr(t["ao_wofs"]), ptr(t["ao_wd"])
    d.weight_entry = ptr(t["w_entry"])
    d.radial_type = int(bt.radial)
    d.ao_kr = ptr(t["ao_kr"])
    d.ao_wv = ptr(t["ao_wv"]) if not bt.contract else None
    if mo is not None:
        scf = dev64(mo.mo_scf, device)
        mod = dev64(mo.mo_modifier, device)
        keep += [scf, mod]
        d.nmo = scf.shape[1]
        d.mo_scf, d.mo_modifier = ptr(scf), ptr(mod)
    else:
        d.nmo = 1
        d.mo_scf = d.mo_modifier = ptr(dd)
    d.nmo_used = d.nmo if nmo_used is None else nmo_used
    ee, en = jastrow_parts(jastrow)
    if ee is not None:
        wj = dev64(ee.jastrow_kernel.weight, device)
        keep.append(wj)
        d.use_jastrow = 1
        d.jastrow_w = ptr(wj)
    else:
        d.use_jastrow = 0
        d.jastrow_w = ptr(dd)
    if en is not None:
        wn = dev64(en.jastrow_kernel.weight, device)
        at = dev64(en.atoms, device).reshape(-1)
        keep += [wn, at]
        d.use_jastrow_en = 1
        d.jastrow_en_w, d.jastrow_en_atoms = ptr(wn), ptr(at)
    else:
        d.use_jastrow_en = 0
        d.jastrow_en_w = d.jastrow_en_atoms = ptr(dd)
    if pool is not None:
        ct = pool.device_tables(device)
        keep.append(ct)
        d.det_mode = 1 if ct.explicit else 0
        d.ncfg = ct.ncfg
        d.max_orb[0], d.max_orb[1] = ct.max_orb
        d.ndet[0], d.ndet[1] = ct.ndet
        d.det_table[0], d.det_table[1] = ptr(ct.t["det_table0"]), ptr(ct.t["det_table1"])
        d.cfg_det[0], d.cfg_det[1] = ptr(ct.t["cfg_det0"]), ptr(ct.t["cfg_det1"])
    else:
        d.det_mode, d.ncfg = 0, 1
        d.max_orb[0], d.max_orb[1] = d.nup, d.ndown
        d.ndet[0] = d.ndet[1] = 1
        d.det_table[0] = d.det_table[1] = ptr(di)
        d.cfg_det[0] = d.cfg_det[1] = ptr(di)
    if fc is not None:
        cw = dev64(fc.weight.reshape(-1), device)
        keep.append(cw)
        d.ci_weight = ptr(cw)
    else:
        d.ci_weight = ptr(dd)
    d.e_nuc = float(e_nuc)
    d.precision = int(precision)
    return Call(d, keep)
