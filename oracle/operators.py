"""Dense Hamiltonian and MPO square (oracle).

Reference: tnpy/operators.py:89-116 (MatrixProductOperator.square),
tnpy/operators.py:119-166 (FullHamiltonian: k0 is the most significant digit
of the row index, :145-154; n*log2(d) <= 12 enforced, :140-143).
"""
from __future__ import annotations

import numpy as np

from .models import uniform


def full_hamiltonian(mpo: list[np.ndarray]) -> np.ndarray:
    """Contract the whole MPO into H[(k0..k_{n-1}), (b0..b_{n-1})]."""
    w = uniform(mpo)
    n = len(w)
    d = w[0].shape[-1]
    if d**n > 2**12:
        raise ResourceWarning(f"Requesting more than {n} sites with physical dim {d}.")
    # t[v, K, B] with K, B the fused ket / bra strings so far (k0 most significant)
    t = w[0][0]  # (D, d, d)
    for s in range(1, n):
        ws = w[s]
        # t[w, K, B] * W[w, v, k, b] -> [v, K, k, B, b]
        nt = np.einsum("wKB,wvkb->vKkBb", t, ws)
        dv, dk, _, db, _ = nt.shape
        t = nt.reshape(dv, dk * ws.shape[2], db * ws.shape[3])
    return t[0]


def mpo_square(mpo: list[np.ndarray]) -> list[np.ndarray]:
    """W2[(w1 w2), (v1 v2), k, b] = sum_m W[w1, v1, k, m] W[w2, v2, m, b] (operators.py:97-116)."""
    w = uniform(mpo)
    n = len(w)
    out = []
    for s, ws in enumerate(w):
        sq = np.einsum("acKm,bdmB->abcdKB", ws, ws)
        a, b, c, dd, k, bb = sq.shape
        sq = sq.reshape(a * b, c * dd, k, bb)
        if s == 0:
            sq = sq[0]
        elif s == n - 1:
            sq = sq[:, 0]
        out.append(sq)
    return out
