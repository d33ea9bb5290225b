"""MPO builders (oracle). Arrays follow the reference's (l, r, k, b) order.

Reference: tnpy/model/xxz.py:8-30, tnpy/model/random_heisenberg.py:8-119,
tnpy/model/utils.py:7-64, tnpy/model/model_1d.py:25-33,
tnpy/operators.py:10-63 (SpinOperators).

The MPO is a list of numpy arrays with the reference's shapes: site 0 is
``W[row]`` of shape (D, d, d), site n-1 is ``W[:, col]`` of shape (D, d, d),
every other site is (D, D, d, d).
"""
from __future__ import annotations

import numpy as np


def spin_operators(spin: float = 0.5):
    """Sp, Sm, Sz, I2, O2 as in tnpy/operators.py:55-60."""
    sp = spin * np.array([[0, 2], [0, 0]], dtype=float)
    sm = spin * np.array([[0, 0], [2, 0]], dtype=float)
    sz = spin * np.array([[1, 0], [0, -1]], dtype=float)
    return sp, sm, sz, np.identity(2, dtype=float), np.zeros((2, 2), dtype=float)


def _boundary(tensor: np.ndarray, site: int, n: int, row: int = 0, col: int = -1):
    """tnpy/model/utils.py:21-29 (boundary_vectors decorator)."""
    if site == 0:
        return tensor[row, :, :, :]
    if site == n - 1:
        return tensor[:, col, :, :]
    return tensor


def xxz_mpo(n: int, delta: float) -> list[np.ndarray]:
    """tnpy/model/xxz.py:19-30: H = sum -1/2 (S+S- + S-S+) - delta SzSz."""
    sp, sm, sz, i2, o2 = spin_operators()
    elem = np.array(
        [
            [i2, -0.5 * sp, -0.5 * sm, -delta * sz, o2],
            [o2, o2, o2, o2, sm],
            [o2, o2, o2, o2, sp],
            [o2, o2, o2, o2, sz],
            [o2, o2, o2, o2, i2],
        ]
    )
    return [_boundary(elem.copy(), s, n) for s in range(n)]


def random_fields(n: int, h: float, seed) -> np.ndarray:
    """tnpy/model/random_heisenberg.py:57-58."""
    return np.random.RandomState(seed).uniform(-h, h, size=n)


def random_heisenberg_mpo(
    n: int, h: float, penalty: float = 0.0, s_target: int = 0, offset: float = 0.0, seed=None
) -> list[np.ndarray]:
    """tnpy/model/random_heisenberg.py:84-109 (with minors_if_no_penalty, utils.py:47-64)."""
    sp, sm, sz, i2, o2 = spin_operators()
    fields = random_fields(n, h, seed)
    out = []
    for site in range(n):
        alpha = penalty * (0.25 + s_target**2 / n) - offset / n
        beta = fields[site] - 2.0 * penalty * s_target
        mat = np.array(
            [
                [i2, 0.5 * sp, 0.5 * sm, 2.0 * penalty * sz, sz, alpha * i2 + beta * sz],
                [o2, o2, o2, o2, o2, sm],
                [o2, o2, o2, o2, o2, sp],
                [o2, o2, o2, i2, o2, sz],
                [o2, o2, o2, o2, o2, sz],
                [o2, o2, o2, o2, o2, i2],
            ],
            dtype=float,
        )
        if penalty == 0:
            mat = np.delete(np.delete(mat, 3, axis=0), 3, axis=1)
        out.append(_boundary(mat, site, n))
    return out


def random_couplings(n: int, delta: float, seed) -> np.ndarray:
    """J_i = (1 - u_i)^(1/delta), u_i ~ U[0, 1) so that 1 - u_i lies in (0, 1].

    Builder addition (the reference has no random-coupling Heisenberg chain);
    the draw uses np.random.RandomState(seed) like random_heisenberg.py:57-58.
    """
    u = np.random.RandomState(seed).uniform(size=n - 1)
    return (1.0 - u) ** (1.0 / delta)


def random_coupling_heisenberg_mpo(
    n: int, couplings: np.ndarray, h: float = 0.0, fields: np.ndarray | None = None
) -> list[np.ndarray]:
    """H = sum_i J_i S_i . S_{i+1} + h_i Sz_i.

    Same D=5 layout as random_heisenberg.py:92-109 with penalty 0; J_i (the bond
    between i and i+1) multiplies the Sp, Sm and Sz entries of row 0 of site i.
    """
    sp, sm, sz, i2, o2 = spin_operators()
    fields = np.zeros(n) if fields is None else np.asarray(fields, dtype=float)
    out = []
    for site in range(n):
        j = couplings[site] if site < n - 1 else 0.0
        mat = np.array(
            [
                [i2, 0.5 * j * sp, 0.5 * j * sm, j * sz, fields[site] * sz],
                [o2, o2, o2, o2, sm],
                [o2, o2, o2, o2, sp],
                [o2, o2, o2, o2, sz],
                [o2, o2, o2, o2, i2],
            ],
            dtype=float,
        )
        out.append(_boundary(mat, site, n))
    return out


def uniform(mpo: list[np.ndarray]) -> list[np.ndarray]:
    """Give every MPO tensor four indices: site 0 -> (1, D, d, d), site n-1 -> (D, 1, d, d).

    This is the layout the device path uses; it is the same operator (the
    reference drops the dummy index instead, matrix_product_state.py:425-430).
    """
    n = len(mpo)
    out = []
    for s, w in enumerate(mpo):
        if w.ndim == 4:
            out.append(w)
        elif s == 0:
            out.append(w[None, ...])
        else:
            out.append(w[:, None, ...])
    return out
