"""Molecule / basis namespace input for the VMC hot path."""
from .molecule import Molecule, build_basis_namespace, norm_gaussian_cartesian, ANGS2BOHR

__all__ = ["Molecule", "build_basis_namespace", "norm_gaussian_cartesian", "ANGS2BOHR"]
