"""Model1D base class (tnpy/model/model_1d.py:8-33)."""
import abc

import numpy as np

from ..operators import MatrixProductOperator


class Model1D(abc.ABC):
    def __init__(self, n: int):
        self._n = n

    @property
    def n(self) -> int:
        return self._n

    @abc.abstractmethod
    def _elem(self, site: int) -> np.ndarray:
        return NotImplemented

    @property
    def mpo(self) -> MatrixProductOperator:
        return MatrixProductOperator([self._elem(site) for site in range(self.n)])
