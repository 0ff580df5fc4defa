"""Restricted Hartree-Fock molecular orbitals on the basis namespace (stands
in for the reference's pyscf calculator, ``qmctorch/scf/calculator/
pyscf.py:88-103``: ``scf.RHF(mol).run()`` in the spherical basis, MOs mapped to
the cartesian AOs with ``cart2sph_coeff``, columns normalised by
``calculator_base.py:36-46``).

Integrals come from ``qmc_scf_one_electron`` / ``qmc_scf_eri`` (host code of
the native library, McMurchie-Davidson) over the AOs exactly as the AO layer
evaluates them, so the SCF orbitals are those of the wave function's own basis
functions. As pyscf does for a basis of spherical shells, the SCF runs in the
span of the real solid harmonics: a cartesian d shell (xx, xy, xz, yy, yz, zz)
contributes its five l = 2 combinations xy, xz, yz, xx - yy, 2zz - xx - yy,
so the number of MOs is the spherical count ``basis.nmo``. Iterations: Fock
build from the full ERI tensor, Pulay DIIS on the commutator FDS - SDF,
canonical orthogonalisation; the initial guess is the extended-Hueckel
density. Closed shells only (``spin = 0``).
"""
from __future__ import annotations

import ctypes

import numpy as np


def gto_arrays(basis, atom_coords):
    """Per-entry arrays of the AO layer's basis functions: function index,
    centre, exponent, weight (coefficient x norm), cartesian powers."""
    centers = np.repeat(np.asarray(atom_coords, dtype=np.float64), basis.nshells, axis=0)
    w = np.asarray(basis.bas_coeffs, dtype=np.float64) * np.asarray(basis.bas_norm,
                                                                    dtype=np.float64)
    k = np.stack([basis.bas_kx, basis.bas_ky, basis.bas_kz], axis=1).astype(np.int32)
    return {"ao": np.ascontiguousarray(np.asarray(basis.index_ctr, dtype=np.int32)),
            "center": np.ascontiguousarray(centers),
            "exp": np.ascontiguousarray(np.asarray(basis.bas_exp, dtype=np.float64)),
            "coef": np.ascontiguousarray(w), "k": np.ascontiguousarray(k)}


def _desc(basis, arrays):
    from .. import _lib
    d = _lib.GtoBasis()
    d.nao = int(basis.nao)
    d.nprim = len(arrays["exp"])
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    d.prim_ao, d.prim_center = ptr(arrays["ao"]), ptr(arrays["center"])
    d.prim_exp, d.prim_coef, d.prim_k = ptr(arrays["exp"]), ptr(arrays["coef"]), ptr(arrays["k"])
    return d


def integrals(basis, atom_coords, charges):
    """(S, T, V, ERI) of the basis, host arrays; ERI[p, q, r, s] = (pq|rs)."""
    from .. import _lib
    lib = _lib.lib()
    arr = gto_arrays(basis, atom_coords)
    d = _desc(basis, arr)
    n = int(basis.nao)
    xyz = np.ascontiguousarray(np.asarray(atom_coords, dtype=np.float64))
    z = np.ascontiguousarray(np.asarray(charges, dtype=np.float64))
    S, T, V = (np.empty((n, n)) for _ in range(3))
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    _lib.check(lib.qmc_scf_one_electron(ctypes.byref(d), len(z), ptr(xyz), ptr(z), ptr(S),
                                        ptr(T), ptr(V)), "qmc_scf_one_electron")
    eri = np.empty((n, n, n, n))
    _lib.check(lib.qmc_scf_eri(ctypes.byref(d), ptr(eri)), "qmc_scf_eri")
    return S, T, V, eri


def spherical_map(basis):
    """(nao_cart, nsph) matrix whose columns span each shell's real solid
    harmonics in the normalised cartesian functions."""
    cols = []
    for (_, lval, a0, ncomp, _) in basis._shell_info:
        if lval < 2:
            for c in range(ncomp):
                v = np.zeros(basis.nao)
                v[a0 + c] = 1.0
                cols.append(v)
            continue
        # components xx, xy, xz, yy, yz, zz at a0 .. a0 + 5 (equal norms on xx, yy, zz)
        for comb in ({1: 1.0}, {2: 1.0}, {4: 1.0}, {0: 1.0, 3: -1.0},
                     {5: 2.0, 0: -1.0, 3: -1.0}):
            v = np.zeros(basis.nao)
            for c, x in comb.items():
                v[a0 + c] = x
            cols.append(v)
    return np.stack(cols, axis=1)


def nuclear_repulsion(atom_coords, charges):
    xyz = np.asarray(atom_coords, dtype=np.float64)
    z = np.asarray(charges, dtype=np.float64)
    e = 0.0
    for a in range(len(z)):
        for b in range(a + 1, len(z)):
            e += z[a] * z[b] / np.linalg.norm(xyz[a] - xyz[b])
    return e


def rhf(basis, atom_coords, charges, nelec, guess=None, max_iter=100, conv=1e-10,
        diis_size=8):
    """Closed-shell RHF: returns (mos (nao_cart, nsph) column-normalised,
    orbital energies, total energy, converged)."""
    if nelec % 2:
        raise ValueError("the RHF calculator handles closed shells (even electron counts)")
    S0, T0, V0, eri0 = integrals(basis, atom_coords, charges)
    C = spherical_map(basis)
    S = C.T @ S0 @ C
    H = C.T @ (T0 + V0) @ C
    n = S.shape[0]
    eri = np.einsum("pqrs,pi,qj,rk,sl->ijkl", eri0, C, C, C, C, optimize=True) \
        if n != basis.nao else eri0
    eri2 = eri.reshape(n * n, n * n)
    erik = np.ascontiguousarray(eri.transpose(0, 2, 1, 3)).reshape(n * n, n * n)
    s, U = np.linalg.eigh(S)
    keep = s > 1e-9 * s.max()
    X = U[:, keep] / np.sqrt(s[keep])
    nocc = nelec // 2
    if guess is not None:
        # least-squares projection of the guess orbitals on the spherical span
        cg = np.linalg.lstsq(C, guess[:, :nocc], rcond=None)[0]
        cg = cg @ np.linalg.inv(np.linalg.cholesky(cg.T @ S @ cg)).T
        D = 2.0 * cg @ cg.T
    else:
        e, Cp = np.linalg.eigh(X.T @ H @ X)
        Co = X @ Cp[:, :nocc]
        D = 2.0 * Co @ Co.T
    enuc = nuclear_repulsion(atom_coords, charges)
    focks, errs = [], []
    e_old, converged = 0.0, False
    for it in range(max_iter):
        J = (eri2 @ D.reshape(-1)).reshape(n, n)
        K = (erik @ D.reshape(-1)).reshape(n, n)
        F = H + J - 0.5 * K
        e_elec = 0.5 * float(np.sum(D * (H + F)))
        err = X.T @ (F @ D @ S - S @ D @ F) @ X
        focks.append(F)
        errs.append(err)
        focks, errs = focks[-diis_size:], errs[-diis_size:]
        if len(focks) > 1:
            m = len(focks)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for i in range(m):
                for j in range(m):
                    B[i, j] = float(np.sum(errs[i] * errs[j]))
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            try:
                cvec = np.linalg.solve(B, rhs)[:m]
                F = sum(c * f for c, f in zip(cvec, focks))
            except np.linalg.LinAlgError:
                pass
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        Cs = X @ Cp
        D = 2.0 * Cs[:, :nocc] @ Cs[:, :nocc].T
        if abs(e_elec - e_old) < conv and np.abs(err).max() < 1e-7:
            converged = True
            break
        e_old = e_elec
    # final orbitals of the converged Fock matrix (no DIIS extrapolation)
    J = (eri2 @ D.reshape(-1)).reshape(n, n)
    K = (erik @ D.reshape(-1)).reshape(n, n)
    F = H + J - 0.5 * K
    e_tot = 0.5 * float(np.sum(D * (H + F))) + enuc
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    mos = C @ (X @ Cp)
    mos = mos / np.sqrt((mos ** 2).sum(0))
    return mos, e, e_tot, converged
