"""Host-side tables the kernels consume: AO groups and CI determinant recipes.

``basis_tables`` turns the basis namespace (one entry per contracted-AO
primitive, ``qmctorch/scf/calculator/pyscf.py:104-252``) into AO *groups*:
consecutive AOs on one atom whose primitive exponents are identical (the
cartesian components of a shell and the columns of a general contraction).
The kernels evaluate one exponential per (electron, group primitive) and reuse
it for every AO of the group.

``config_tables`` turns the CI configurations into per-spin determinant
recipes with the index conventions of the reference pooling layer:
``get_unique_excitation`` (``orbital_configurations.py:357-402``),
``ExcitationMask.get_index_unique_single/double``
(``orbital_projector.py:126-189``, including the use of the spin-up
excitation for the spin-down double indices, line 186) and
``OrbitalProjector.get_unique_configs`` (``orbital_projector.py:29-51``).
"""
from __future__ import annotations

import math
from itertools import combinations, product

import numpy as np
import torch

_DF = {-1: 1, 0: 1, 1: 1, 2: 2, 3: 3, 5: 15, 7: 105}
MAX_COMP = 6


def norm_cst(bas_kx, bas_ky, bas_kz, bas_exp):
    """Per-entry cartesian GTO norm, computed once from the namespace
    exponents as in ``atomic_orbital_norm`` (norm_orbital.py:136-161,
    atomic_orbitals.py:93-94)."""
    a = np.asarray(bas_exp, dtype=np.float64)
    out = (2.0 * a / np.pi) ** 0.75
    for k in (bas_kx, bas_ky, bas_kz):
        k = np.asarray(k)
        df = np.array([_DF[int(2 * v - 1)] for v in k], dtype=np.float64)
        out = out * (4.0 * a) ** (k / 2.0) / np.sqrt(df)
    return out


def _dfact(n):
    out = 1
    for k in range(int(n), 0, -2):
        out *= k
    return out


def norm_slater_cst(bas_kx, bas_ky, bas_kz, bas_kr, bas_exp):
    """Per-entry norm of a cartesian STO x^a y^b z^c r^n exp(-alpha r)
    (``norm_slater_cartesian``, norm_orbital.py:106-161): with
    L = a + b + c + n + 1, 1 / sqrt(4 pi (2L)! / (2 alpha)^(2L + 1)
    (2a-1)!! (2b-1)!! (2c-1)!! / (2a + 2b + 2c + 1)!!)."""
    a, b, c = (np.asarray(v, dtype=np.int64) for v in (bas_kx, bas_ky, bas_kz))
    n = np.asarray(bas_kr, dtype=np.float64)
    alpha = np.asarray(bas_exp, dtype=np.float64)
    lv = a + b + c + n + 1.0
    lfact = np.array([float(math.factorial(int(2 * v))) for v in lv])
    pref = 4.0 * np.pi * lfact / (2.0 * alpha) ** (2.0 * lv + 1.0)
    num = np.array([float(_dfact(2 * x - 1) * _dfact(2 * y - 1) * _dfact(2 * z - 1))
                    for x, y, z in zip(a, b, c)])
    den = np.array([float(_dfact(2 * x + 2 * y + 2 * z + 1)) for x, y, z in zip(a, b, c)])
    return np.sqrt(1.0 / (pref * num / den))


RADIAL = {"gto": 0, "gto_pure": 0, "sto": 1, "sto_pure": 2}


def entry_norms(basis):
    """The AO layer's per-entry norms (atomic_orbital_norm, norm_orbital.py:8-47)
    for the cartesian radial types this package evaluates."""
    if str(basis.radial_type).startswith("sto"):
        kr = getattr(basis, "bas_kr", np.zeros(len(basis.bas_exp)))
        return norm_slater_cst(basis.bas_kx, basis.bas_ky, basis.bas_kz, kr, basis.bas_exp)
    return norm_cst(basis.bas_kx, basis.bas_ky, basis.bas_kz, basis.bas_exp)


class BasisTables:
    """AO group tables built from the namespace and the current exponents."""

    def __init__(self, basis, bas_exp_values):
        if basis.harmonics_type != "cart" or str(basis.radial_type) not in RADIAL:
            raise NotImplementedError(
                "the GB300 AO kernels evaluate cartesian harmonics with Gaussian (pyscf layout) "
                "or Slater (ADF layout) radial functions")
        self.radial = RADIAL[str(basis.radial_type)]
        self.nao = int(basis.nao)
        index_ctr = np.asarray(basis.index_ctr, dtype=np.int64)
        nshells = np.asarray(basis.nshells, dtype=np.int64)
        entry_atom = np.repeat(np.arange(len(nshells)), nshells)
        kxyz = np.stack([np.asarray(basis.bas_kx), np.asarray(basis.bas_ky),
                         np.asarray(basis.bas_kz)], axis=1).astype(np.int64)
        coeffs = np.asarray(basis.bas_coeffs, dtype=np.float64)
        norm = entry_norms(basis)
        kr = np.asarray(getattr(basis, "bas_kr", np.zeros(len(index_ctr))), dtype=np.int64)
        if self.radial != 1:
            kr = np.zeros_like(kr)
        self.contract = len(np.unique(index_ctr)) != len(index_ctr)
        exps = np.asarray(bas_exp_values, dtype=np.float64)
        # entries of each AO, in namespace order
        ao_entries = [[] for _ in range(self.nao)]
        for e, a in enumerate(index_ctr):
            ao_entries[a].append(e)
        ao_atom = np.zeros(self.nao, dtype=np.int64)
        ao_k = np.zeros((self.nao, 3), dtype=np.int64)
        ao_kr = np.zeros(self.nao, dtype=np.int64)
        for a, ents in enumerate(ao_entries):
            if not ents:
                raise ValueError("AO %d has no primitive" % a)
            at = set(entry_atom[ents].tolist())
            ks = {tuple(kxyz[e]) for e in ents}
            krs = {int(kr[e]) for e in ents}
            if len(at) != 1 or len(ks) != 1 or len(krs) != 1:
                raise NotImplementedError("AO %d mixes atoms or powers" % a)
            ao_atom[a] = at.pop()
            ao_k[a] = ks.pop()
            ao_kr[a] = krs.pop()
        # group consecutive AOs with identical exponent lists on the same atom
        groups = []
        a = 0
        while a < self.nao:
            key = exps[ao_entries[a]].tobytes()
            b = a + 1
            while (b < self.nao and b - a < MAX_COMP and ao_atom[b] == ao_atom[a]
                   and exps[ao_entries[b]].tobytes() == key and ao_kr[b] == ao_kr[a]):
                b += 1
            groups.append((a, b))
            a = b
        group_atom, group_prim, group_ao, gprim_entry = [], [0], [0], []
        ao_wofs = np.zeros(self.nao, dtype=np.int64)
        wd, wv, w_entry = [], [], []
        for (a0, a1) in groups:
            ents0 = ao_entries[a0]
            group_atom.append(int(ao_atom[a0]))
            gprim_entry += ents0
            group_prim.append(group_prim[-1] + len(ents0))
            group_ao.append(a1)
            for a in range(a0, a1):
                ao_wofs[a] = len(wd)
                for e in ao_entries[a]:
                    wd.append(coeffs[e] * norm[e])
                    wv.append(norm[e])
                    w_entry.append(e)
        self.group_key = [exps[ao_entries[a0]].tobytes() for (a0, _) in groups]
        self.groups = groups
        self.ao_entries = ao_entries
        i32 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.int32))  # noqa: E731
        f64 = lambda x: torch.as_tensor(np.asarray(x, dtype=np.float64))  # noqa: E731
        self.t = {
            "group_atom": i32(group_atom), "group_prim": i32(group_prim),
            "group_ao": i32(group_ao), "gprim_entry": i32(gprim_entry),
            "ao_k": i32(ao_k.reshape(-1)), "ao_wofs": i32(ao_wofs), "ao_wd": f64(wd),
            "ao_wv": f64(wv), "w_entry": i32(w_entry), "ao_kr": i32(ao_kr),
        }
        self.ngroup = len(groups)
        self.ngprim = len(gprim_entry)
        self.nweight = len(wd)
        self.nentries = len(index_ctr)

    def still_valid(self, bas_exp_values):
        """True while every AO of a group keeps the group's exponents."""
        exps = np.asarray(bas_exp_values, dtype=np.float64)
        for (a0, a1), key in zip(self.groups, self.group_key):
            for a in range(a0, a1):
                if exps[self.ao_entries[a]].tobytes() != key:
                    return False
        return True

    def to(self, device):
        self.t = {k: v.to(device) for k, v in self.t.items()}
        return self


# ----------------------------------------------------------------------------
# CI configurations
# ----------------------------------------------------------------------------
class OrbitalConfigurations:
    """``OrbitalConfigurations`` (orbital_configurations.py:6-312)."""

    def __init__(self, mol):
        self.nup = mol.nup
        self.ndown = mol.ndown
        self.nelec = self.nup + self.ndown
        self.spin = getattr(mol, "spin", 0)
        self.norb = mol.basis.nmo

    def get_configs(self, configs):
        if isinstance(configs, str):
            configs = configs.lower()
        if isinstance(configs, tuple):
            assert len(configs) == 2
            assert configs[0].shape == configs[1].shape
            assert len(configs[0][0]) == self.nup
            assert len(configs[0][0]) == self.ndown
            return configs
        if configs == "ground_state":
            return (torch.LongTensor([list(range(self.nup))]),
                    torch.LongTensor([list(range(self.ndown))]))
        for prefix in ("cas", "single_double", "single"):
            if configs.startswith(prefix + "("):
                nelec, norb = (int(v) for v in configs[len(prefix) + 1:].rstrip(")").split(","))
                break
        else:
            raise ValueError("Config error: %s not recognized as valid configuration" % configs)
        if nelec > self.nelec:
            raise ValueError("required number of electron in config too large")
        if norb > self.norb:
            raise ValueError("required number of orbitals in config too large")
        nocc = (nelec // 2, nelec // 2) if nelec % 2 == 0 else (nelec // 2 + 1, nelec // 2)
        nvirt = (norb - nocc[0], norb - nocc[1])
        if prefix == "cas":
            return self._cas(nocc, nvirt, nelec)
        cup, cdn = self._singles(nocc, nvirt)
        if prefix == "single":
            return torch.LongTensor(cup), torch.LongTensor(cdn)
        return self._single_double(cup, cdn, nocc, nvirt)

    def _singles(self, nocc, nvirt):
        gs_up, gs_dn = list(range(self.nup)), list(range(self.ndown))
        cup, cdn = [gs_up], [gs_dn]
        for io in range(self.nup - 1, self.nup - 1 - nocc[0], -1):
            for iv in range(self.nup, self.nup + nvirt[0]):
                x = gs_up.copy()
                x[io] = iv
                cup.append(x)
                cdn.append(gs_dn)
        for io in range(self.ndown - 1, self.ndown - 1 - nocc[1], -1):
            for iv in range(self.ndown, self.ndown + nvirt[1]):
                x = gs_dn.copy()
                x[io] = iv
                cup.append(gs_up)
                cdn.append(x)
        return cup, cdn

    def _single_double(self, cup, cdn, nocc, nvirt):
        gs_up, gs_dn = list(range(self.nup)), list(range(self.ndown))
        occ_up = list(range(self.nup - 1, self.nup - 1 - nocc[0], -1))
        vrt_up = list(range(self.nup, self.nup + nvirt[0]))
        occ_dn = list(range(self.ndown - 1, self.ndown - 1 - nocc[1], -1))
        vrt_dn = list(range(self.ndown, self.ndown + nvirt[1]))
        for ou in occ_up:
            for vu in vrt_up:
                for od in occ_dn:
                    for vd in vrt_dn:
                        xu, xd = gs_up.copy(), gs_dn.copy()
                        xu[ou] = vu
                        xd[od] = vd
                        cup.append(xu)
                        cdn.append(xd)
        for o1, o2 in combinations(occ_up, 2):
            for v1, v2 in combinations(vrt_up, 2):
                x = gs_up.copy()
                x[o1] = v2
                x[o2] = v1
                cup.append(x)
                cdn.append(gs_dn)
        for o1, o2 in combinations(occ_dn, 2):
            for v1, v2 in combinations(vrt_dn, 2):
                x = gs_dn.copy()
                x[o1] = v2
                x[o2] = v1
                cup.append(gs_up)
                cdn.append(x)
        return torch.LongTensor(cup), torch.LongTensor(cdn)

    def _cas(self, nocc, nvirt, nelec):
        if self.spin != 0:
            raise ValueError("CAS active space not possible with spin polarized calculation")
        lo, hi = self.nup - nocc[0], self.nup + nvirt[0]
        frz = list(range(lo))
        cu = [frz + list(c) for c in combinations(range(lo, hi), nelec // 2)]
        cd = [frz + list(c) for c in combinations(range(lo, hi), nelec // 2)]
        conf = list(product(cu, cd))
        return torch.LongTensor([c[0] for c in conf]), torch.LongTensor([c[1] for c in conf])


def get_unique_excitation(configs):
    """``get_unique_excitation`` (orbital_configurations.py:357-402)."""
    uu, ud, iu, idn = [], [], [], []
    for ic, (cu, cd) in enumerate(zip(configs[0], configs[1])):
        su, sd = set(tuple(cu.tolist())), set(tuple(cd.tolist()))
        if ic == 0:
            gu, gd = su, sd
        eu = [list(gu.difference(su)), list(su.difference(gu))]
        ed = [list(gd.difference(sd)), list(sd.difference(gd))]
        if eu not in uu:
            uu.append(eu)
        if ed not in ud:
            ud.append(ed)
        iu.append(uu.index(eu))
        idn.append(ud.index(ed))
    return (uu, ud), (iu, idn)


class ConfigTables:
    """Per-spin determinant recipes for the kernels."""

    def __init__(self, config_method, configs, nup, ndown):
        self.method = config_method
        cu = torch.as_tensor(configs[0])
        cd = torch.as_tensor(configs[1])
        self.ncfg = int(cu.shape[0])
        self.max_orb = (int(cu.max()) + 1, int(cd.max()) + 1)
        explicit = config_method.startswith("cas(") or config_method == "explicit"
        self.explicit = explicit
        if explicit:
            ucu, icu = torch.unique(cu, dim=0, return_inverse=True)
            ucd, icd = torch.unique(cd, dim=0, return_inverse=True)
            tabs = [ucu.reshape(-1), ucd.reshape(-1)]
            self.ndet = (int(ucu.shape[0]), int(ucd.shape[0]))
            cfg = [icu.reshape(-1), icd.reshape(-1)]
        else:
            (uu, ud), (iu, idn) = get_unique_excitation((cu, cd))
            ncu, ncd = self.max_orb[0] - nup, self.max_orb[1] - ndown
            su, sd, du, dd = [], [], [], []
            for eu, ed in zip(uu, ud):
                if len(eu[0]) == 1:
                    su.append(eu[0][0] * ncu + eu[1][0] - nup)
                if len(ed[1]) == 1:
                    sd.append(ed[0][0] * ncd + ed[1][0] - ndown)
            for eu, ed in zip(uu, ud):
                if len(eu[0]) == 2:
                    for ie in eu[0]:
                        for io in eu[1]:
                            du.append(ie * ncu + io - nup)
                if len(ed[1]) == 2:
                    for ie in eu[0]:  # orbital_projector.py:186 reads exc_up
                        for io in eu[1]:
                            dd.append(ie * ncd + io - ndown)
            do_single = len(su) != 0
            do_double = len(du) != 0
            tabs, nd = [], []
            for singles, doubles in ((su, du), (sd, dd)):
                rows = [[0, 0, 0, 0, 0]]
                if config_method != "ground_state":
                    if do_single:
                        rows += [[1, i, 0, 0, 0] for i in singles]
                    if do_double:
                        rows += [[2] + doubles[4 * k:4 * k + 4] for k in range(len(doubles) // 4)]
                tabs.append(torch.as_tensor(np.asarray(rows, dtype=np.int64).reshape(-1)))
                nd.append(len(rows))
            self.ndet = tuple(nd)
            cfg = [torch.as_tensor(iu), torch.as_tensor(idn)]
            for s in range(2):
                if int(cfg[s].max()) >= self.ndet[s]:
                    raise ValueError("configuration set not supported by the excitation pooling")
        self.t = {"det_table0": tabs[0].to(torch.int32), "det_table1": tabs[1].to(torch.int32),
                  "cfg_det0": cfg[0].to(torch.int32), "cfg_det1": cfg[1].to(torch.int32)}

    def to(self, device):
        self.t = {k: v.to(device) for k, v in self.t.items()}
        return self
