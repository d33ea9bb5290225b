"""Tree-tensor-network SDRG (oracle), restating tnpy/tsdrg.py:444-696.

MPO tensors are kept in the uniform (Dl, Dr, m, m) layout; the reference's
``isel`` of row 0 / column -1 on four-index tensors (tsdrg.py:621-625) is then
``W1[0]`` / ``W2[:, -1]`` for every tensor (a no-op on the one-sized dummy
index of the boundary tensors).
"""
from __future__ import annotations

import numpy as np

from .models import uniform


def block_hamiltonian(w1: np.ndarray, w2: np.ndarray) -> np.ndarray:
    """H[(k1 k2), (b1 b2)] = sum_w W1[0, w, k1, b1] W2[w, -1, k2, b2] (tsdrg.py:607-631)."""
    a = w1[0]  # (w, k1, b1)
    b = w2[:, -1]  # (w, k2, b2)
    h = np.einsum("wkb,wKB->kKbB", a, b)
    m1, m2 = a.shape[1], b.shape[1]
    return h.reshape(m1 * m2, m1 * m2)


def block_eigen_solver(h: np.ndarray, chi: int):
    """Full eigh, keep the lowest chi pairs (tsdrg.py:569-592; its debug prints dropped)."""
    evals, evecs = np.linalg.eigh(h)
    if h.shape[0] > chi:
        evals, evecs = evals[:chi], evecs[:, :chi]
    return evals, evecs


def truncation_gap(evals: np.ndarray, chi: int) -> float:
    """tsdrg.py:594-605, including its behaviour on already-truncated spectra: ``evals`` has
    at most chi entries, so the gap is always evals[-1] - evals[-2]."""
    gaps = np.diff(evals)
    return float(gaps[chi - 1] if gaps.size > chi else gaps[-1])


def spectrum_projector(w1: np.ndarray, w2: np.ndarray, evecs: np.ndarray):
    """W'[l, r, i, j] = sum W1[l,w,k1,b1] W2[w,r,k2,b2] V[k1,k2,i] V[b1,b2,j] (tsdrg.py:633-669).

    Returns (W', V) with V of shape (m1, m2, k).
    """
    m1, m2 = w1.shape[2], w2.shape[2]
    v = evecs.reshape(m1, m2, evecs.shape[1])
    t = np.einsum("lwkb,wrKB->lrkKbB", w1, w2)
    t = np.einsum("lrkKbB,kKi->lribB", t, v)
    t = np.einsum("lribB,bBj->lrij", t, v)
    return t, v


class TreeTensorNetworkSDRG:
    def solve(self, h: np.ndarray):
        return block_eigen_solver(h, self.chi)

    def gap_of(self, evals: np.ndarray) -> float:
        return truncation_gap(evals, self.chi)

    def __init__(self, mpo, chi: int):
        self.chi = chi
        self.n = len(mpo)
        self.cache = [w.copy() for w in uniform(mpo)]
        self.horizon = list(range(self.n))
        self.merges: list[tuple[int, int, int]] = []
        self.projectors: dict[int, np.ndarray] = {}
        self.evals = None
        self.gap: list[float] = []
        self.evecs: list[np.ndarray] = []
        for bond in range(self.n - 1):
            ev, vec = self.solve(block_hamiltonian(self.cache[bond], self.cache[bond + 1]))
            self.evecs.append(vec)
            self.gap.append(self.gap_of(ev))
            self.evals = ev if self.n == 2 else None

    def _neighbours(self, bond: int):
        """tsdrg.py:463-479 (evaluated after the merged tensor is popped)."""
        if bond == 0:
            return [bond]
        if bond == len(self.cache) - 1:
            return [bond - 1]
        return [bond - 1, bond]

    def run(self):
        """tsdrg.py:671-696: merge the bond with the largest gap (first on ties)."""
        step = 0
        while True:
            step += 1
            b = int(np.argmax(np.array(self.gap)))
            new_id = self.n + step - 1
            w_new, v = spectrum_projector(self.cache[b], self.cache[b + 1], self.evecs[b])
            self.merges.append((self.horizon[b], self.horizon[b + 1], new_id))
            self.projectors[new_id] = v
            self.cache.pop(b + 1)
            self.cache[b] = w_new
            self.horizon[b] = new_id
            self.horizon.pop(b + 1)
            if len(self.cache) == 1:
                break
            self.gap.pop(b)
            self.evecs.pop(b)
            for bond in self._neighbours(b):
                ev, vec = self.solve(block_hamiltonian(self.cache[bond], self.cache[bond + 1]))
                self.gap[bond] = self.gap_of(ev)
                self.evecs[bond] = vec
                self.evals = ev
        return self


class HighEnergyTreeTensorNetworkSDRG(TreeTensorNetworkSDRG):
    """tsdrg.py:1031-1067: keep the chi highest pairs; gap evals[-chi] - evals[-chi-1], or the
    first gap of a spectrum with at most chi gaps."""

    def solve(self, h: np.ndarray):
        evals, evecs = np.linalg.eigh(h)
        if h.shape[0] > self.chi:
            evals, evecs = evals[-self.chi:], evecs[:, -self.chi:]
        return evals, evecs

    def gap_of(self, evals: np.ndarray) -> float:
        gaps = np.diff(evals)
        return float(gaps[-self.chi] if gaps.size > self.chi else gaps[0])


class ShiftInvertTreeTensorNetworkSDRG(TreeTensorNetworkSDRG):
    """tsdrg.py:1070-1089: generalised eigh(H, H^2) (eigenvalues 1/E), keep the chi smallest,
    report 1/lambda + offset in ascending order with the vectors H x (unit norm)."""

    def __init__(self, mpo, chi: int, offset: float):
        self.offset = offset
        super().__init__(mpo, chi)

    def solve(self, h: np.ndarray):
        import scipy.linalg as spl

        evals, evecs = spl.eigh(h, b=h @ h)
        if h.shape[0] > self.chi:
            evals, evecs = evals[: self.chi], evecs[:, : self.chi]
        evals = np.reciprocal(evals) + self.offset
        idx = np.argsort(evals)
        return evals[idx], h @ evecs[:, idx]
