"""Molecule and basis namespace: the input side of the VMC hot path.

The AO layer of QMCTorch consumes a ``mol.basis`` namespace produced by its
SCF calculator (``qmctorch/scf/calculator/pyscf.py:104-252``). pyscf is not
available on the machines this package targets, so :class:`Molecule` builds
the same namespace from the built-in basis tables (``basis_tables.py``) with
the same entry layout:

* one *entry* per (shell, general contraction, cartesian component,
  primitive), in pyscf shell order (``pyscf.py:146-203``);
* general-contraction column ``ictr`` divided by ``ictr + 1``
  (``pyscf.py:172``);
* cartesian component order ``xx, xy, xz, yy, yz, zz`` for d shells
  (``pyscf.py:120-122``);
* ``nshells`` = number of entries per atom, ``index_ctr`` = AO index of each
  entry, ``nao_per_atom``, ``nctr_per_ao`` (``pyscf.py:206-223``);
* ``mos`` column-normalised (``calculator_base.py:36-46``).

Molecular orbitals: ``calculator="pyscf"`` (the reference's default) runs
this package's restricted Hartree-Fock (``rhf.py``: native McMurchie-Davidson
integrals over the AOs as the AO layer evaluates them, SCF in the span of the
real solid harmonics like pyscf's spherical basis); ``calculator="huckel"``
(or ``"builtin"``) keeps the extended-Hueckel guess (Wolfsberg-Helmholz,
K = 1.75) on the overlap matrix, which is also the SCF's starting density.
``nmo`` is the reference's count of spherical MOs (a d shell contributes 5).
SCF results are cached per (atoms, coordinates, basis) for the process.
"""
from __future__ import annotations

import itertools
import math
from types import SimpleNamespace

import numpy as np

from .basis_tables import ATOMIC_NUMBER, BASIS_TABLES, HUCKEL_VSIE

ANGS2BOHR = 1.8897259886  # qmctorch/utils/constants.py:1

_KX = {0: [0], 1: [1, 0, 0], 2: [2, 1, 1, 0, 0, 0]}
_KY = {0: [0], 1: [0, 1, 0], 2: [0, 1, 0, 2, 1, 0]}
_KZ = {0: [0], 1: [0, 0, 1], 2: [0, 0, 1, 0, 1, 2]}
_MV = {0: [0], 1: [-1, 0, 1], 2: [-2, -1, 0, 1, 2]}
_DFACT = {-1: 1, 0: 1, 1: 1, 2: 2, 3: 3, 5: 15}


def norm_gaussian_cartesian(kx, ky, kz, alpha):
    """Per-entry norm of a cartesian GTO, as the AO layer computes it
    (``qmctorch/wavefunction/orbitals/norm_orbital.py:136-161``):
    (2a/pi)^(3/4) * prod_i (4a)^(k_i/2) / sqrt((2k_i-1)!!)."""
    kx = np.asarray(kx)
    ky = np.asarray(ky)
    kz = np.asarray(kz)
    alpha = np.asarray(alpha, dtype=np.float64)
    pref = (2.0 * alpha / np.pi) ** 0.75
    out = pref
    for k in (kx, ky, kz):
        df = np.array([_DFACT[int(2 * v - 1)] for v in k], dtype=np.float64)
        out = out * (4.0 * alpha) ** (k / 2.0) / np.sqrt(df)
    return out


def build_basis_namespace(atoms, atom_coords, basis_name):
    """Lay out the basis entries the way ``CalculatorPySCF.get_basis_data``
    does (``qmctorch/scf/calculator/pyscf.py:104-252``)."""
    table = BASIS_TABLES[basis_name.lower()]
    natm = len(atoms)
    nshells = [0] * natm
    bas_coeff, bas_exp, index_ctr = [], [], []
    bas_l, bas_m, bas_n, bas_kx, bas_ky, bas_kz = [], [], [], [], [], []
    shell_info = []  # (atom, l, first AO, ncomp, role) for the Hueckel guess
    iao = 0
    for iat, sym in enumerate(atoms):
        seen_s = 0
        for lval, exps, coeffs in table[sym]:
            coeffs = np.asarray(coeffs, dtype=np.float64)
            exps = np.asarray(exps, dtype=np.float64)
            nprim, nctr = coeffs.shape
            ncart = len(_KX[lval])
            for ictr in range(nctr):
                cc = coeffs[:, ictr] / (ictr + 1)
                bas_coeff += cc.tolist() * ncart
                bas_exp += exps.tolist() * ncart
                bas_l += [lval] * nprim * ncart
                bas_n += [lval + 1] * nprim * ncart
                nshells[iat] += nprim * ncart
                if lval == 0:
                    role = 0 if (seen_s == 0 and ATOMIC_NUMBER[sym] > 2) else 1
                    seen_s += 1
                else:
                    role = 1 + lval
                shell_info.append((iat, lval, iao, ncart, role))
                for _ in range(ncart):
                    index_ctr += [iao] * nprim
                    iao += 1
                for m in _MV[lval]:
                    bas_m += [m] * nprim
                for k in _KX[lval]:
                    bas_kx += [k] * nprim
                for k in _KY[lval]:
                    bas_ky += [k] * nprim
                for k in _KZ[lval]:
                    bas_kz += [k] * nprim

    basis = SimpleNamespace()
    basis.radial_type = "gto_pure"
    basis.harmonics_type = "cart"
    basis.nao = iao
    nsph = 0
    for (_, lval, _, _, _) in shell_info:
        nsph += 2 * lval + 1
    basis.nmo = nsph
    basis.nshells = nshells
    basis.index_ctr = index_ctr
    intervals = np.concatenate(([0], np.cumsum(nshells)))
    basis.nao_per_atom = [
        len(np.unique(index_ctr[intervals[i]:intervals[i + 1]])) for i in range(natm)
    ]
    basis.nctr_per_ao = np.array([len(list(g)) for _, g in itertools.groupby(index_ctr)])
    basis.bas_coeffs = np.array(bas_coeff)
    basis.bas_exp = np.array(bas_exp)
    basis.bas_n = bas_n
    basis.bas_l = bas_l
    basis.bas_m = bas_m
    basis.bas_kr = np.zeros_like(basis.bas_exp)
    basis.bas_kx = np.array(bas_kx)
    basis.bas_ky = np.array(bas_ky)
    basis.bas_kz = np.array(bas_kz)
    basis.bas_norm = norm_gaussian_cartesian(basis.bas_kx, basis.bas_ky, basis.bas_kz,
                                             basis.bas_exp)
    basis.atom_coords_internal = np.asarray(atom_coords, dtype=np.float64)
    basis.TotalEnergy = float("nan")
    basis._shell_info = shell_info
    return basis


def _overlap_1d_table(kmax, xpa, xpb, inv2p):
    """Obara-Saika 1D overlap recursion for arrays of primitive pairs:
    table[a][b] (a, b <= kmax), each an array over the pairs."""
    s = [[None] * (kmax + 1) for _ in range(kmax + 1)]
    s[0][0] = np.ones_like(xpa)
    for a in range(kmax + 1):
        for b in range(kmax + 1):
            if a == 0 and b == 0:
                continue
            if a > 0:
                v = xpa * s[a - 1][b] if b <= kmax else None
                if a > 1:
                    v = v + inv2p * (a - 1) * s[a - 2][b]
                if b > 0:
                    v = v + inv2p * b * s[a - 1][b - 1]
            else:
                v = xpb * s[a][b - 1]
                if b > 1:
                    v = v + inv2p * (b - 1) * s[a][b - 2]
            s[a][b] = v
    return s


def ao_overlap(basis, atom_coords):
    """Overlap matrix of the AOs as evaluated by the AO layer
    (weights c_p * N_p, entries summed by index_ctr); all primitive pairs at
    once."""
    nao = basis.nao
    centers = np.repeat(np.asarray(atom_coords, dtype=np.float64), basis.nshells, axis=0)
    w = np.asarray(basis.bas_coeffs, dtype=np.float64) * np.asarray(basis.bas_norm)
    k = np.stack([basis.bas_kx, basis.bas_ky, basis.bas_kz], axis=1).astype(np.int64)
    idx = np.asarray(basis.index_ctr, dtype=np.int64)
    ex = np.asarray(basis.bas_exp, dtype=np.float64)
    p, q = np.triu_indices(len(w))
    a, b = ex[p], ex[q]
    A, B = centers[p], centers[q]
    pp = a + b
    P = (a[:, None] * A + b[:, None] * B) / pp[:, None]
    dAB = (A - B) ** 2
    r2 = -a * b / pp * ((dAB[:, 0] + dAB[:, 1]) + dAB[:, 2])
    # scalar libm exp / pow per pair (array versions may round differently)
    val = np.array([math.exp(x) * (math.pi / y) ** 1.5 for x, y in zip(r2.tolist(), pp.tolist())])
    kmax = int(k.max()) if k.size else 0
    for d in range(3):
        tab = _overlap_1d_table(kmax, P[:, d] - A[:, d], P[:, d] - B[:, d], 0.5 / pp)
        sd = np.empty_like(val)
        for ka in range(kmax + 1):
            for kb in range(kmax + 1):
                m = (k[p, d] == ka) & (k[q, d] == kb)
                sd[m] = tab[ka][kb][m]
        val = val * sd
    val = val * (w[p] * w[q])
    # accumulate in pair order, (p, q) then (q, p), so that S is summed exactly
    # as a loop over the pairs would
    off = p != q
    n = len(p)
    rows = np.stack([idx[p], np.where(off, idx[q], -1)], axis=1).reshape(-1)
    cols = np.stack([idx[q], np.where(off, idx[p], -1)], axis=1).reshape(-1)
    vals = np.stack([val, val], axis=1).reshape(-1)
    keep = rows >= 0
    S = np.zeros((nao, nao))
    np.add.at(S, (rows[keep], cols[keep]), vals[keep])
    return S


def huckel_mos(basis, atoms, atom_coords, k_wh=1.75):
    """Extended-Hueckel MOs (lowest ``basis.nmo`` eigenvectors of H C = S C E)."""
    import scipy.linalg

    S = ao_overlap(basis, atom_coords)
    hdiag = np.zeros(basis.nao)
    for (iat, lval, a0, ncomp, role) in basis._shell_info:
        hdiag[a0:a0 + ncomp] = HUCKEL_VSIE[atoms[iat]][min(role, 3)]
    H = k_wh * S * 0.5 * (hdiag[:, None] + hdiag[None, :])
    np.fill_diagonal(H, hdiag * np.diag(S))
    evals, evecs = scipy.linalg.eigh(H, S)
    mos = evecs[:, : basis.nmo]
    # pyscf.py:247 + calculator_base.py:36-46: plain column 2-norm
    mos = mos / np.sqrt((mos ** 2).sum(0))
    return mos, evals[: basis.nmo]


# Minimal Slater-type basis ("slater-sz") with exponents from Slater's rules
# (J. C. Slater, Phys. Rev. 36, 57 (1930)): zeta = (Z - s) / n with the
# screening s of the rules; shells (n, l) per element, a 3d polarisation
# shell (zeta 2.0) on second-row atoms. In the ADF layout the AO layer reads:
# cartesian powers kx, ky, kz and the power of r, kr = n - 1 - l.
SLATER_SZ = {
    "H": [(1, 0, 1.0)],
    "Li": [(1, 0, 2.70), (2, 0, 0.65), (2, 1, 0.65)],
    "C": [(1, 0, 5.70), (2, 0, 1.625), (2, 1, 1.625), (3, 2, 2.0)],
    "O": [(1, 0, 7.70), (2, 0, 2.275), (2, 1, 2.275), (3, 2, 2.0)],
}


def build_slater_namespace(atoms, atom_coords, seed=0):
    """Basis namespace of the ADF calculator's layout (adf.py:205-275:
    radial_type "sto", cartesian harmonics, one uncontracted entry per AO,
    coefficients 1) for the "slater-sz" basis. No Slater-orbital integrals
    are available here, so the MOs are seeded orthonormal columns (synthetic
    inputs of the right shape), normalised as the reference does."""
    from ..wavefunction.tables import norm_slater_cst
    nshells, kx, ky, kz, kr, ex, bn, bl = [], [], [], [], [], [], [], []
    for sym in atoms:
        cnt = 0
        for (n, lval, zeta) in SLATER_SZ[sym]:
            for c in range(len(_KX[lval])):
                kx.append(_KX[lval][c])
                ky.append(_KY[lval][c])
                kz.append(_KZ[lval][c])
                kr.append(n - 1 - lval)
                ex.append(zeta)
                bn.append(n)
                bl.append(lval)
                cnt += 1
        nshells.append(cnt)
    nao = len(ex)
    basis = SimpleNamespace()
    basis.radial_type = "sto"
    basis.harmonics_type = "cart"
    basis.nao = nao
    basis.nmo = nao
    basis.nshells = nshells
    basis.nao_per_atom = nshells
    basis.index_ctr = np.arange(nao)
    basis.nctr_per_ao = np.ones(nao, dtype=np.int64)
    basis.bas_kx, basis.bas_ky, basis.bas_kz = (np.array(v) for v in (kx, ky, kz))
    basis.bas_kr = np.array(kr)
    basis.bas_exp = np.array(ex, dtype=np.float64)
    basis.bas_coeffs = np.ones(nao)
    basis.bas_n, basis.bas_l = bn, bl
    basis.bas_m = [0] * nao
    basis.bas_norm = norm_slater_cst(basis.bas_kx, basis.bas_ky, basis.bas_kz, basis.bas_kr,
                                     basis.bas_exp)
    basis.atom_coords_internal = np.asarray(atom_coords, dtype=np.float64)
    q, _ = np.linalg.qr(np.random.default_rng(seed).normal(size=(nao, nao)))
    basis.mos = q / np.sqrt((q ** 2).sum(0))
    basis.mo_energy = np.arange(nao, dtype=np.float64)
    basis.TotalEnergy = float("nan")
    return basis


_SCF_CACHE = {}


def scf_orbitals(basis, atoms, atom_coords, charges, nelec):
    """RHF orbitals of the namespace (cached): (mos, mo_energy, total energy)."""
    from .rhf import rhf
    key = (tuple(atoms), tuple(np.round(np.asarray(atom_coords, dtype=np.float64), 12).ravel()),
           basis.nao, basis.nmo, tuple(np.round(basis.bas_exp, 12)), nelec)
    if key not in _SCF_CACHE:
        guess, _ = huckel_mos(basis, atoms, atom_coords)
        mos, mo_energy, etot, converged = rhf(basis, atom_coords, charges, nelec, guess=guess)
        if not converged:
            raise RuntimeError("RHF did not converge for %s" % "".join(atoms))
        if len(_SCF_CACHE) > 256:
            _SCF_CACHE.clear()
        _SCF_CACHE[key] = (mos, mo_energy, etot)
    mos, mo_energy, etot = _SCF_CACHE[key]
    return mos.copy(), mo_energy.copy(), etot


class Molecule:
    """Drop-in for ``qmctorch.scf.Molecule`` (``qmctorch/scf/molecule.py:22-162``)
    restricted to what the hot path reads: ``nelec, nup, ndown, spin, natom,
    atoms, atomic_number, atomic_nelec, atom_coords, hdf5file, basis``.

    ``calculator``: ``"pyscf"`` (default, RHF orbitals as the reference's pyscf
    calculator provides them, computed by this package) or ``"huckel"`` /
    ``"builtin"`` (extended-Hueckel guess), both on the built-in Gaussian
    tables; ``"slater"``: the minimal Slater-type basis "slater-sz" in the ADF
    calculator's layout with synthetic orthonormal MOs.
    ``load`` accepts a ``.npz`` file written by :meth:`save`.
    """

    def __init__(self, atom=None, calculator="pyscf", scf="hf", basis="sto-3g",
                 unit="bohr", charge=0, spin=0, name=None, load=None,
                 save_scf_file=False, redo_scf=False, rank=0, mpi_size=0):
        self.atom_coords = []
        self.atomic_nelec = []
        self.atomic_number = []
        self.atoms = []
        self.charge = charge
        self.spin = spin
        self.unit = unit
        self.name = name
        self.basis_name = basis
        self.calculator_name = calculator
        self.scf_level = scf
        self.nelec = 0
        if load is not None:
            self._load_npz(load)
            return
        if unit not in ("angs", "bohr"):
            raise ValueError("unit should be angs or bohr")
        if calculator not in ("pyscf", "builtin", "huckel", "slater"):
            raise ValueError("calculator must be 'pyscf' (RHF), 'huckel' or 'slater'")
        for a in atom.split(";"):
            if not a.strip():
                continue
            data = a.split()
            sym = data[0]
            conv = ANGS2BOHR if unit == "angs" else 1.0
            self.atoms.append(sym)
            self.atom_coords.append([float(data[1]) * conv, float(data[2]) * conv,
                                     float(data[3]) * conv])
            z = ATOMIC_NUMBER[sym]
            self.atomic_number.append(z)
            self.atomic_nelec.append(z)
            self.nelec += z
        self.nelec += charge
        self.natom = len(self.atoms)
        if (self.nelec - self.spin) % 2 != 0:
            raise ValueError("%d electrons and spin %d doesn't make sense"
                             % (self.nelec, self.spin))
        self.nup = int((self.nelec - self.spin) / 2) + self.spin
        self.ndown = int((self.nelec - self.spin) / 2)
        if self.name is None:
            self.name = "".join(self.atoms)
        self.hdf5file = "_".join([self.name, calculator, basis]) + ".hdf5"
        if calculator == "slater":
            self.basis = build_slater_namespace(self.atoms, self.atom_coords)
            self.atoms = np.array(self.atoms)
            return
        self.basis = build_basis_namespace(self.atoms, self.atom_coords, basis)
        if calculator == "pyscf" and self.spin == 0:
            self.basis.mos, self.basis.mo_energy, self.basis.TotalEnergy = scf_orbitals(
                self.basis, self.atoms, self.atom_coords, self.atomic_number, self.nelec)
        else:
            self.basis.mos, self.basis.mo_energy = huckel_mos(self.basis, self.atoms,
                                                              self.atom_coords)
        self.atoms = np.array(self.atoms)

    def domain(self, method):
        """Walker initialisation domains (``qmctorch/scf/molecule.py:176-214``)."""
        domain = {"method": method}
        if method == "center":
            domain["center"] = np.mean(self.atom_coords, 0)
        elif method == "uniform":
            domain["min"] = np.min(self.atom_coords) - 0.5
            domain["max"] = np.max(self.atom_coords) + 0.5
        elif method == "normal":
            domain["mean"] = np.mean(self.atom_coords, 0)
            domain["sigma"] = np.diag(np.std(self.atom_coords, 0) + 0.25)
        elif method == "atomic":
            domain["atom_coords"] = self.atom_coords
            domain["atom_num"] = self.atomic_number
            domain["atom_nelec"] = self.atomic_nelec
        else:
            raise ValueError("Method to initialize the walkers not recognized")
        return domain

    _BASIS_KEYS = ("nao", "nmo", "nshells", "index_ctr", "nao_per_atom", "nctr_per_ao",
                   "bas_coeffs", "bas_exp", "bas_n", "bas_l", "bas_m", "bas_kr", "bas_kx",
                   "bas_ky", "bas_kz", "bas_norm", "atom_coords_internal", "mos", "TotalEnergy")

    def save(self, filename):
        """Write the molecule and its basis namespace to ``.npz``."""
        data = {"mol_" + k: np.asarray(getattr(self, k)) for k in
                ("atoms", "atom_coords", "atomic_number", "atomic_nelec", "nelec", "nup",
                 "ndown", "spin", "charge")}
        for k in self._BASIS_KEYS:
            data["basis_" + k] = np.asarray(getattr(self.basis, k))
        data["basis_radial_type"] = np.asarray(self.basis.radial_type)
        data["basis_harmonics_type"] = np.asarray(self.basis.harmonics_type)
        np.savez(filename, **data)

    def _load_npz(self, filename):
        with np.load(filename, allow_pickle=False) as f:
            self.atoms = f["mol_atoms"].astype("U")
            self.atom_coords = f["mol_atom_coords"].tolist()
            self.atomic_number = [int(x) for x in f["mol_atomic_number"]]
            self.atomic_nelec = [int(x) for x in f["mol_atomic_nelec"]]
            self.nelec = int(f["mol_nelec"])
            self.nup = int(f["mol_nup"])
            self.ndown = int(f["mol_ndown"])
            self.spin = int(f["mol_spin"])
            self.charge = int(f["mol_charge"])
            self.natom = len(self.atoms)
            self.basis = SimpleNamespace()
            for k in self._BASIS_KEYS:
                v = f["basis_" + k]
                setattr(self.basis, k, v.item() if v.ndim == 0 else v)
            self.basis.nao = int(self.basis.nao)
            self.basis.nmo = int(self.basis.nmo)
            self.basis.radial_type = str(f["basis_radial_type"])
            self.basis.harmonics_type = str(f["basis_harmonics_type"])
        self.name = self.name or "".join(self.atoms)
        self.hdf5file = filename
