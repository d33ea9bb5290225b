"""Exact diagonalisation (oracle), tnpy/exact_diagonalization.py:10-60."""
from __future__ import annotations

import numpy as np

from .operators import full_hamiltonian


class ExactDiagonalization:
    def __init__(self, mpo):
        self.matrix = full_hamiltonian(mpo)
        self.evals, self.evecs = np.linalg.eigh(self.matrix)
