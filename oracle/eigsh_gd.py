"""Davidson GD+1 eigensolver in numpy (oracle / CPU baseline -- test infrastructure only).

Restates the eigensolver behind ``linalg.eigshmv`` (tnpy/linalg.py:64-87):
``primme.eigsh(A, k=1, which='SA', v0, tol)`` of PRIMME 3.2.1 (a C library pinned in the
reference's poetry.lock, absent here). PRIMME's default method family is the generalised
Davidson method with thick restarting and "+k" locally optimal restarting (GD+k; Stathopoulos
& McCombs, ACM TOMS 37 (2010) 21). For one wanted pair and no preconditioner (the reference
passes none, so the correction is the residual itself) that is:

* basis V (orthonormal, classical Gram-Schmidt with one reorthogonalisation), AV = A V, the
  projected matrix H = V^T A V and its lowest Ritz pair (theta, y), x = V y;
* convergence when ||A x - theta x|| <= tol * ||A||, with ||A|| estimated as the largest
  |Ritz value| seen (PRIMME's estimate when the caller gives no norm);
* at max_basis vectors, restart to [x, x_prev orthogonalised against x] (GD+1: the previous
  step's Ritz vector is kept, which makes the restarted iteration locally optimal).

The scipy ARPACK restatement in ``dmrg.eigsh_lowest`` stays the parity oracle (run at a
tight tolerance); this one models the reference's matvec count at the reference's tolerance,
which is what a timed CPU baseline needs.
"""
from __future__ import annotations

import numpy as np


def eigsh_gd(op, v0: np.ndarray, tol: float = 1e-8, max_basis: int = 24, max_matvecs: int = 2000):
    """Lowest eigenpair of the symmetric operator ``op`` (a function of a flat vector).

    Returns (theta, x, matvecs, converged) with x of unit norm."""
    n = v0.size
    mb = max(2, min(max_basis, n))
    V = np.empty((mb, n))
    AV = np.empty((mb, n))
    H = np.zeros((mb, mb))
    t = np.asarray(v0, dtype=float).reshape(-1).copy()
    k = mv = 0
    anorm = 0.0
    theta, x = 0.0, t / max(np.linalg.norm(t), 1e-300)
    y_prev = None
    while True:
        for _ in range(2):  # CGS2 against the basis
            if k:
                t -= V[:k].T @ (V[:k] @ t)
        nt = np.linalg.norm(t)
        if not nt > 1e-14 * max(1.0, np.linalg.norm(x)):
            return theta, x, mv, False  # the correction fell inside the basis
        V[k] = t / nt
        AV[k] = op(V[k])
        mv += 1
        col = V[: k + 1] @ AV[k]
        H[: k + 1, k] = col
        H[k, : k + 1] = col
        k += 1
        w, s = np.linalg.eigh(H[:k, :k])
        theta, y = float(w[0]), s[:, 0]
        anorm = max(anorm, float(np.abs(w).max()))
        x = y @ V[:k]
        r = y @ AV[:k] - theta * x
        if np.linalg.norm(r) <= tol * anorm or k >= n:
            return theta, x, mv, True
        if mv >= max_matvecs:
            return theta, x, mv, False
        if k == mb:
            keep = [y]
            if y_prev is not None and y_prev.size == k - 1:
                yp = np.append(y_prev, 0.0)
                yp -= (y @ yp) * y
                if np.linalg.norm(yp) > 1e-6:
                    keep.append(yp / np.linalg.norm(yp))
            S = np.stack(keep, 1)  # (k, m)
            V[: S.shape[1]] = (S.T @ V[:k])
            AV[: S.shape[1]] = (S.T @ AV[:k])
            Hs = S.T @ H[:k, :k] @ S
            k = S.shape[1]
            H[:] = 0.0
            H[:k, :k] = 0.5 * (Hs + Hs.T)
            y_prev = None
        else:
            y_prev = y
        t = r
