from .metropolis import Metropolis, SamplerBase, Walkers

__all__ = ["Metropolis", "SamplerBase", "Walkers"]
