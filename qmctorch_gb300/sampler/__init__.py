from .generalized_metropolis import GeneralizedMetropolis
from .metropolis import Metropolis, SamplerBase, Walkers

__all__ = ["GeneralizedMetropolis", "Metropolis", "SamplerBase", "Walkers"]
