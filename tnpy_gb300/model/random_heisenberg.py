"""Random-field Heisenberg chain (tnpy/model/random_heisenberg.py:8-119) and the
random-coupling chain used for batched tSDRG."""
from __future__ import annotations

import numpy as np

from ..operators import SpinOperators
from .model_1d import Model1D
from .utils import boundary_vectors, minors_if_no_penalty


class RandomHeisenberg(Model1D):
    """H = sum S_i.S_{i+1} + h_i Sz_i, h_i ~ U[-h, h) from RandomState(seed) (:57-58),
    optional penalty lambda (sum Sz - s_target)^2 and offset."""

    def __init__(self, n: int, h: float, penalty: float = 0, s_target: int = 0, offset: float = 0,
                 trial_id: str | None = None, seed: int | None = None):
        super().__init__(n)
        self._h = h
        self._penalty = penalty
        self._s_target = s_target
        self._offset = offset
        self._trial_id = trial_id
        self._seed = seed
        self._random_sequence = np.random.RandomState(seed).uniform(-h, h, size=n)

    @property
    def h(self) -> float:
        return self._h

    @property
    def penalty(self) -> float:
        return self._penalty

    @property
    def s_target(self) -> int:
        return self._s_target

    @property
    def offset(self) -> float:
        return self._offset

    @offset.setter
    def offset(self, offset: float):
        self._offset = offset

    @property
    def trial_id(self):
        return self._trial_id

    @property
    def seed(self):
        return self._seed

    @seed.setter
    def seed(self, seed: int) -> None:
        self._seed = seed
        self._random_sequence = np.random.RandomState(seed).uniform(-self.h, self.h, size=self.n)

    @boundary_vectors(row=0, col=-1)
    @minors_if_no_penalty(row=3, col=3)
    def _elem(self, site: int) -> np.ndarray:
        Sp, Sm, Sz, I2, O2 = SpinOperators()
        alpha = self.penalty * (0.25 + self.s_target**2 / self.n) - self.offset / self.n
        beta = self._random_sequence[site] - 2.0 * self.penalty * self.s_target
        return np.array(
            [
                [I2, 0.5 * Sp, 0.5 * Sm, 2.0 * self.penalty * Sz, Sz, alpha * I2 + beta * Sz],
                [O2, O2, O2, O2, O2, Sm],
                [O2, O2, O2, O2, O2, Sp],
                [O2, O2, O2, I2, O2, Sz],
                [O2, O2, O2, O2, O2, Sz],
                [O2, O2, O2, O2, O2, I2],
            ],
            dtype=float,
        )


class RandomCouplingHeisenberg(Model1D):
    """H = sum_i J_i S_i.S_{i+1} + h_i Sz_i with J_i = (1 - u_i)^(1/delta),
    u_i ~ U[0, 1) from RandomState(seed) (so J_i in (0, 1]); fields h_i ~ U[-h, h)
    from RandomState(seed + 1) when h > 0. The reference has no random-coupling
    chain; the MPO keeps the D=5 layout of RandomHeisenberg with J_i on the
    Sp, Sm and Sz entries of row 0."""

    def __init__(self, n: int, delta: float = 1.0, h: float = 0.0, seed: int | None = None):
        super().__init__(n)
        self.delta = delta
        self.h = h
        self.seed = seed
        u = np.random.RandomState(seed).uniform(size=n - 1)
        self.couplings = (1.0 - u) ** (1.0 / delta)
        self.fields = (np.random.RandomState(None if seed is None else seed + 1).uniform(-h, h, size=n)
                       if h > 0 else np.zeros(n))

    @boundary_vectors(row=0, col=-1)
    def _elem(self, site: int) -> np.ndarray:
        Sp, Sm, Sz, I2, O2 = SpinOperators()
        j = self.couplings[site] if site < self.n - 1 else 0.0
        return np.array(
            [
                [I2, 0.5 * j * Sp, 0.5 * j * Sm, j * Sz, self.fields[site] * Sz],
                [O2, O2, O2, O2, Sm],
                [O2, O2, O2, O2, Sp],
                [O2, O2, O2, O2, Sz],
                [O2, O2, O2, O2, I2],
            ],
            dtype=float,
        )
