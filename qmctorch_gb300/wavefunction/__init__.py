from .slater_jastrow import SlaterJastrow, WaveFunction
from .jastrows import JastrowFactorElectronElectron, PadeJastrowKernel
from .orbitals import AtomicOrbitals, MolecularOrbitals
from .pooling import SlaterPooling
from .tables import OrbitalConfigurations

__all__ = ["SlaterJastrow", "WaveFunction", "JastrowFactorElectronElectron", "PadeJastrowKernel",
           "AtomicOrbitals", "MolecularOrbitals", "SlaterPooling", "OrbitalConfigurations"]
