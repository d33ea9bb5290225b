"""XXZ chain, H = sum -1/2 (S+S- + S-S+) - delta SzSz (tnpy/model/xxz.py:8-30).

The antiferromagnetic chain sum SxSx + SySy + 0.5 SzSz is XXZ(n, delta=-0.5)
(same spectrum and <Sz_i> on an open chain, by a pi rotation of every second
spin about z).
"""
import numpy as np

from ..operators import SpinOperators
from .model_1d import Model1D
from .utils import boundary_vectors


class XXZ(Model1D):
    def __init__(self, n: int, delta: float):
        super().__init__(n)
        self.delta = delta

    @boundary_vectors(row=0, col=-1)
    def _elem(self, site: int) -> np.ndarray:
        Sp, Sm, Sz, I2, O2 = SpinOperators()
        return np.array(
            [
                [I2, -0.5 * Sp, -0.5 * Sm, -self.delta * Sz, O2],
                [O2, O2, O2, O2, Sm],
                [O2, O2, O2, O2, Sp],
                [O2, O2, O2, O2, Sz],
                [O2, O2, O2, O2, I2],
            ]
        )
