"""Spin operators, the MPO container and the dense Hamiltonian.

Reference: tnpy/operators.py:10-166. The MPO is host-side input (small FP64
arrays in the reference's (l, r, k, b) order, site 0 as W[row] and site n-1 as
W[:, col]); ``device_tensors`` gives the uniform four-index device copies the
kernels take (1-sized dl on site 0 and dr on site n-1).
"""
from __future__ import annotations

from dataclasses import InitVar, astuple, dataclass, field

import numpy as np
import torch


@dataclass
class SpinOperators:
    """Sp, Sm, Sz, I2, O2 (tnpy/operators.py:10-63); unpack in that order."""

    spin: InitVar[float] = field(default=0.5)
    Sp: np.ndarray = field(init=False)
    Sm: np.ndarray = field(init=False)
    Sz: np.ndarray = field(init=False)
    I2: np.ndarray = field(init=False)
    O2: np.ndarray = field(init=False)

    def __post_init__(self, spin: float):
        self.Sp = spin * np.array([[0, 2], [0, 0]], dtype=float)
        self.Sm = spin * np.array([[0, 0], [2, 0]], dtype=float)
        self.Sz = spin * np.array([[1, 0], [0, -1]], dtype=float)
        self.I2 = np.identity(2, dtype=float)
        self.O2 = np.zeros((2, 2), dtype=float)

    def __iter__(self):
        return iter(astuple(self))


class MatrixProductOperator:
    """List of MPO tensors (tnpy/operators.py:66-116)."""

    def __init__(self, arrays):
        self._arrays = [np.ascontiguousarray(np.asarray(a, dtype=float)) for a in arrays]
        n = len(self._arrays)
        if n < 2:
            raise ValueError("an MPO needs at least two sites")
        phys = {a.shape[-1] for a in self._arrays} | {a.shape[-2] for a in self._arrays}
        if len(phys) != 1:
            raise ValueError("All MPO tensors are assumed to have same physical dims.")
        self._phys_dim = phys.pop()
        self._device_cache: dict = {}

    @property
    def n_sites(self) -> int:
        return len(self._arrays)

    nsites = n_sites

    @property
    def phys_dim(self) -> int:
        return self._phys_dim

    def __len__(self):
        return len(self._arrays)

    def __getitem__(self, site: int) -> np.ndarray:
        return self._arrays[site]

    def __iter__(self):
        return iter(self._arrays)

    def uniform(self) -> list[np.ndarray]:
        """Four-index tensors: site 0 -> (1, D, d, d), site n-1 -> (D, 1, d, d)."""
        out = []
        for s, w in enumerate(self._arrays):
            if w.ndim == 4:
                out.append(w)
            elif s == 0:
                out.append(w[None])
            else:
                out.append(w[:, None])
        return out

    def device_tensors(self, device=None) -> list[torch.Tensor]:
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        key = str(dev)
        if key not in self._device_cache:
            self._device_cache[key] = [torch.from_numpy(np.ascontiguousarray(w)).to(dev) for w in self.uniform()]
        return self._device_cache[key]

    def __mul__(self, c):
        arrays = [a.copy() for a in self._arrays]
        arrays[0] = c * arrays[0]
        return MatrixProductOperator(arrays)

    __rmul__ = __mul__

    def square(self) -> "MatrixProductOperator":
        """Bilayer MPO of H^2 (operators.py:89-116): W2[(w1 w2),(v1 v2),k,b] = sum_m W[w1,v1,k,m] W[w2,v2,m,b]."""
        n = self.n_sites
        out = []
        for s, w in enumerate(self.uniform()):
            sq = np.einsum("acKm,bdmB->abcdKB", w, w)
            a, b, c, d, k, bb = sq.shape
            sq = sq.reshape(a * b, c * d, k, bb)
            out.append(sq[0] if s == 0 else sq[:, 0] if s == n - 1 else sq)
        return MatrixProductOperator(out)


class FullHamiltonian:
    """Dense H with k0 as the most significant digit (tnpy/operators.py:119-166).

    Host-side, for n*log2(d) <= 12 as in the reference (:140-143)."""

    def __init__(self, mpo: MatrixProductOperator):
        self._n_sites = mpo.n_sites
        self._phys_dim = mpo.phys_dim
        if self.phys_dim**self.n_sites > 2**12:
            raise ResourceWarning(
                f"Requesting more than {self.n_sites} sites with physical dim {self.phys_dim}."
            )
        w = mpo.uniform()
        t = w[0][0]
        for ws in w[1:]:
            nt = np.einsum("wKB,wvkb->vKkBb", t, ws)
            t = nt.reshape(nt.shape[0], nt.shape[1] * nt.shape[2], nt.shape[3] * nt.shape[4])
        self._matrix = t[0]

    @property
    def n_sites(self) -> int:
        return self._n_sites

    @property
    def phys_dim(self) -> int:
        return self._phys_dim

    @property
    def matrix(self) -> np.ndarray:
        return self._matrix
