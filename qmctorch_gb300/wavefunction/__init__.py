from .slater_jastrow import SlaterJastrow, WaveFunction
from .jastrows import (CombineJastrow, JastrowFactorElectronElectron, JastrowFactorElectronNuclei,
                       PadeJastrowKernel, PadeJastrowKernelElectronNuclei)
from .orbitals import AtomicOrbitals, MolecularOrbitals
from .pooling import SlaterPooling
from .tables import OrbitalConfigurations

__all__ = ["SlaterJastrow", "WaveFunction", "JastrowFactorElectronElectron", "PadeJastrowKernel",
           "JastrowFactorElectronNuclei", "PadeJastrowKernelElectronNuclei", "CombineJastrow",
           "AtomicOrbitals", "MolecularOrbitals", "SlaterPooling", "OrbitalConfigurations"]
