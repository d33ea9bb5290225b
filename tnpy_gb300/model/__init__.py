from .model_1d import Model1D
from .random_heisenberg import RandomCouplingHeisenberg, RandomHeisenberg
from .xxz import XXZ

__all__ = ["Model1D", "XXZ", "RandomHeisenberg", "RandomCouplingHeisenberg"]
