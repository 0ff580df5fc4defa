"""Jastrow factors (``qmctorch/wavefunction/jastrows/``): the electron-electron
and electron-nucleus Pade factors and their product."""
from .combine_jastrow import CombineJastrow
from .elec_elec import JastrowFactorElectronElectron, PadeJastrowKernel
from .elec_nuclei import JastrowFactorElectronNuclei
from .elec_nuclei import PadeJastrowKernel as PadeJastrowKernelElectronNuclei

__all__ = ["CombineJastrow", "JastrowFactorElectronElectron", "PadeJastrowKernel",
           "JastrowFactorElectronNuclei", "PadeJastrowKernelElectronNuclei"]
