"""CPU tests of the restricted Hartree-Fock calculator that stands in for the
reference's pyscf calculator (qmctorch/scf/calculator/pyscf.py:88-103).

Known answers: H2 in the STO-3G basis at R = 1.4 bohr, the worked example of
Szabo & Ostlund, "Modern Quantum Chemistry" (1989), section 3.5.2: overlap
0.6593, kinetic 0.7600 / 0.2365, nuclear attraction (both nuclei)
-1.8804 / -1.1948, two-electron integrals (11|11) 0.7746, (11|22) 0.5697,
(12|12) 0.2970, orbital energies -0.578 / 0.670 and total energy -1.1167 Ha
(all to the 4 decimals printed there). Beyond that the checks are
properties: the native overlap equals the independent numpy overlap of the
AO layer's functions, the 8-fold ERI symmetry, the converged Fock matrix has
no occupied-virtual block (Brillouin), the MOs are S-orthogonal, and the
energy is invariant under a rigid translation of the molecule.
"""
import numpy as np
import pytest

from qmctorch_gb300.scf.molecule import (ANGS2BOHR, Molecule, ao_overlap,
                                         build_basis_namespace, huckel_mos)
from qmctorch_gb300.scf.rhf import integrals, rhf, spherical_map


def test_h2_sto3g_textbook_values():
    xyz = [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]]
    b = build_basis_namespace(["H", "H"], xyz, "sto-3g")
    S, T, V, eri = integrals(b, xyz, [1, 1])
    np.testing.assert_allclose(S, [[1.0, 0.6593], [0.6593, 1.0]], atol=5e-5)
    np.testing.assert_allclose(T, [[0.7600, 0.2365], [0.2365, 0.7600]], atol=5e-5)
    np.testing.assert_allclose(V, [[-1.8804, -1.1948], [-1.1948, -1.8804]], atol=5e-5)
    assert abs(eri[0, 0, 0, 0] - 0.7746) < 5e-5
    assert abs(eri[0, 0, 1, 1] - 0.5697) < 5e-5
    assert abs(eri[0, 1, 0, 1] - 0.2970) < 5e-5
    mos, e, etot, conv = rhf(b, xyz, [1, 1], 2)
    assert conv
    np.testing.assert_allclose(e, [-0.578, 0.670], atol=5e-4)
    assert abs(etot - (-1.1167)) < 5e-5


@pytest.fixture(scope="module")
def water():
    xyz = (np.array([[0, 0, 0.1173], [0, 0.7572, -0.4692], [0, -0.7572, -0.4692]])
           * ANGS2BOHR).tolist()
    atoms = ["O", "H", "H"]
    b = build_basis_namespace(atoms, xyz, "cc-pvdz")
    return atoms, xyz, b, integrals(b, xyz, [8, 1, 1])


def test_native_overlap_equals_the_ao_layer_overlap(water):
    atoms, xyz, b, (S, T, V, eri) = water
    np.testing.assert_allclose(S, ao_overlap(b, xyz), rtol=0, atol=1e-12)


def test_eri_symmetry(water):
    atoms, xyz, b, (S, T, V, eri) = water
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        np.testing.assert_allclose(eri, eri.transpose(perm), rtol=0, atol=1e-13)
    np.testing.assert_allclose(T, T.T, atol=1e-13)
    np.testing.assert_allclose(V, V.T, atol=1e-13)


def test_water_rhf_is_stationary_and_orthonormal(water):
    atoms, xyz, b, (S0, T0, V0, eri) = water
    guess, _ = huckel_mos(b, atoms, xyz)
    mos, e, etot, conv = rhf(b, xyz, [8, 1, 1], 10, guess=guess)
    assert conv and mos.shape == (b.nao, b.nmo)
    # RHF/cc-pVDZ of water near its equilibrium geometry is about -76.03 Ha
    assert -76.04 < etot < -76.02
    C = mos / np.sqrt(np.einsum("pi,pq,qi->i", mos, S0, mos))  # S-normalised columns
    np.testing.assert_allclose(C.T @ S0 @ C, np.eye(b.nmo), atol=1e-8)
    D = 2.0 * C[:, :5] @ C[:, :5].T
    J = np.einsum("pqrs,rs->pq", eri, D)
    K = np.einsum("prqs,rs->pq", eri, D)
    F = T0 + V0 + J - 0.5 * K
    Fmo = C.T @ F @ C
    assert np.abs(Fmo[:5, 5:]).max() < 1e-6       # no occupied-virtual coupling
    np.testing.assert_allclose(np.diag(Fmo), e, atol=1e-6)
    # the spherical span: 24 functions for 25 cartesian ones (one d shell)
    assert spherical_map(b).shape == (25, 24)


def test_energy_is_translation_invariant():
    xyz = [[0.0, 0.0, 0.0], [0.0, 0.0, 3.0]]
    shifted = [[0.3, -1.2, 0.7], [0.3, -1.2, 3.7]]
    e = []
    for x in (xyz, shifted):
        b = build_basis_namespace(["Li", "H"], x, "sto-3g")
        e.append(rhf(b, x, [3, 1], 4)[2])
    assert abs(e[0] - e[1]) < 1e-9


def test_molecule_uses_rhf_orbitals_by_default():
    m = Molecule("H 0 0 -0.37; H 0 0 0.37", unit="angs", basis="sto-3g")
    h = Molecule("H 0 0 -0.37; H 0 0 0.37", unit="angs", basis="sto-3g", calculator="huckel")
    assert np.isfinite(m.basis.TotalEnergy) and m.basis.TotalEnergy < -1.11
    assert np.allclose(np.sqrt((m.basis.mos ** 2).sum(0)), 1.0)  # plain column norms
    assert h.basis.mos.shape == m.basis.mos.shape
    with pytest.raises(ValueError):
        Molecule("H 0 0 0; H 0 0 1", calculator="adf")
