from .generalized_metropolis import GeneralizedMetropolis
from .hamiltonian import Hamiltonian
from .metropolis import Metropolis, SamplerBase, Walkers

__all__ = ["GeneralizedMetropolis", "Hamiltonian", "Metropolis", "SamplerBase", "Walkers"]
