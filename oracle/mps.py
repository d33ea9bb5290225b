"""MPS, environments, effective Hamiltonian (oracle).

Uniform layout: every MPS tensor is (chi_l, d, chi_r) ('lpr',
matrix_product_state.py:45) with chi = 1 on the open ends, every MPO tensor
is (Dl, Dr, d, d) (see ``models.uniform``), and environments are
(ket, mpo, bra) with the trivial (1, 1, 1) tensor of ones on the open ends.
This is the same operator as the reference, which drops the dummy indices
instead (matrix_product_state.py:306-307, :327-328, :383-395, :425-430).
"""
from __future__ import annotations

import numpy as np


def bond_dims(n: int, chi: int, d: int = 2) -> list[int]:
    """Bond sizes min(d^i, chi, d^(n-i)) of a compressed random MPS.

    Pinned by tests/test_matrix_product_state.py:11-37 of the reference.
    Returns n+1 values with 1 at both ends.
    """
    return [int(min(d**i, chi, d ** (n - i))) if 0 < i < n else 1 for i in range(n + 1)]


def random_mps(n: int, chi: int, d: int = 2, seed: int = 1234) -> list[np.ndarray]:
    """Seeded N(0,1) MPS, right-canonicalised and normalised.

    Stands in for the unseeded quimb ``MPS_rand_state(...).compress()`` of
    matrix_product_state.py:170-185: same bond sizes; the orthogonality centre
    sits on site 0, where the first (rightward) sweep of FiniteDMRG.run starts.
    """
    rng = np.random.RandomState(seed)
    dims = bond_dims(n, chi, d)
    mps = [rng.standard_normal((dims[i], d, dims[i + 1])) for i in range(n)]
    return right_canonicalize(mps)


def right_canonicalize(mps: list[np.ndarray]) -> list[np.ndarray]:
    mps = [a.copy() for a in mps]
    for i in range(len(mps) - 1, 0, -1):
        cl, d, cr = mps[i].shape
        q, r = np.linalg.qr(mps[i].reshape(cl, d * cr).T)  # M^T = Q R -> M = R^T Q^T
        k = q.shape[1]
        mps[i] = q.T.reshape(k, d, cr)
        mps[i - 1] = np.tensordot(mps[i - 1], r.T, axes=([2], [0]))
        # unit norm at every step (a product of ~n random tensors overflows on long chains)
        mps[i - 1] = mps[i - 1] / np.linalg.norm(mps[i - 1])
    return mps


def update_left(left: np.ndarray, a: np.ndarray, w: np.ndarray) -> np.ndarray:
    """L'[c, v, c'] = sum L[a, w, a'] A[a, s, c] W[w, v, s, s'] A[a', s', c'] (mps.py:296-315)."""
    t1 = np.tensordot(left, a, axes=([0], [0]))  # (w, a', s, c)
    t2 = np.tensordot(t1, w, axes=([0, 2], [0, 2]))  # (a', c, v, s')
    return np.tensordot(t2, a, axes=([0, 3], [0, 1]))  # (c, v, c')


def update_right(right: np.ndarray, a: np.ndarray, w: np.ndarray) -> np.ndarray:
    """R'[a, w, a'] = sum R[c, v, c'] A[a, s, c] W[w, v, s, s'] A[a', s', c'] (mps.py:317-336)."""
    t1 = np.tensordot(a, right, axes=([2], [0]))  # (a, s, v, c')
    t2 = np.tensordot(t1, w, axes=([1, 2], [2, 1]))  # (a, c', w, s')
    return np.tensordot(t2, a, axes=([1, 3], [2, 1]))  # (a, w, a')


def one_site_matvec(left, w, right, x):
    """y[a', s', c'] = sum L[a,w,a'] x[a,s,c] W[w,v,s,s'] R[c,v,c'] (mps.py:411-440)."""
    t1 = np.tensordot(left, x, axes=([0], [0]))  # (w, a', s, c)
    t2 = np.tensordot(t1, w, axes=([0, 2], [0, 2]))  # (a', c, v, s')
    y = np.tensordot(t2, right, axes=([1, 2], [0, 1]))  # (a', s', c')
    return y


def one_site_full_matrix(left, w, right) -> np.ndarray:
    """H[(a, s, c), (a', s', c')] = L[a,w,a'] W[w,v,s,s'] R[c,v,c'] (mps.py:372-409).

    Row = ket indices [L.ket, W.k, R.ket], column = bra indices (the fuse map
    of mps.py:385-408).
    """
    h = np.einsum("awx,wvst,cvy->ascxty", left, w, right)
    n = left.shape[0] * w.shape[2] * right.shape[0]
    return h.reshape(n, n)


def one_site_diagonal(left, w, right) -> np.ndarray:
    """diag(H_eff)[a, s, c] = sum_{w,v} L[a,w,a] W[w,v,s,s] R[c,v,c] (Davidson preconditioner)."""
    ld = np.einsum("awa->aw", left)
    wd = np.einsum("wvss->wvs", w)
    rd = np.einsum("cvc->cv", right)
    return np.einsum("aw,wvs,cv->asc", ld, wd, rd)


def svd(matrix: np.ndarray, cutoff: int):
    """linalg.py:9-23."""
    u, s, vt = np.linalg.svd(matrix, full_matrices=False)
    return u[:, :cutoff], s[:cutoff], vt[:cutoff, :]


def qr(matrix: np.ndarray, cutoff: int):
    """linalg.py:26-39."""
    q, r = np.linalg.qr(matrix, mode="reduced")
    return q[:, :cutoff], r[:cutoff, :]


def split_tensor(mps: list[np.ndarray], site: int, rightward: bool) -> np.ndarray:
    """SVD gauge move, in place (matrix_product_state.py:187-225).

    Rightward: psi (chi_l d, chi_r) = U S V^T, A_site = U, A_{site+1} <- (S V^T) A_{site+1}.
    Leftward:  psi (chi_l, d chi_r) = U S V^T, A_site = V^T, A_{site-1} <- A_{site-1} (U S).
    S V^T / U S are not renormalised. Returns the singular values.
    """
    a = mps[site]
    cl, d, cr = a.shape
    if rightward:
        u, s, vt = svd(a.reshape(cl * d, cr), cutoff=cr)
        mps[site] = u.reshape(cl, d, cr)
        mps[site + 1] = np.tensordot(np.diag(s) @ vt, mps[site + 1], axes=([1], [0]))
    else:
        u, s, vt = svd(a.reshape(cl, d * cr), cutoff=cl)
        mps[site] = vt.reshape(cl, d, cr)
        mps[site - 1] = np.tensordot(mps[site - 1], u @ np.diag(s), axes=([2], [0]))
    return s


class Environment:
    """Left / right environments of an MPS under an MPO (matrix_product_state.py:231-440)."""

    def __init__(self, mpo: list[np.ndarray], mps: list[np.ndarray]):
        from .models import uniform

        self.w = uniform(mpo)
        self.mps = mps
        self.n = len(mps)
        one = np.ones((1, 1, 1))
        self.left = {0: one}
        self.right = {self.n - 1: one}
        for site in range(1, self.n):
            self.update_left(site)
        for site in range(self.n - 2, -1, -1):
            self.update_right(site)

    def update_left(self, site):
        self.left[site] = update_left(self.left[site - 1], self.mps[site - 1], self.w[site - 1])

    def update_right(self, site):
        self.right[site] = update_right(self.right[site + 1], self.mps[site + 1], self.w[site + 1])

    def update(self, site, rightward: bool):
        """matrix_product_state.py:338-353."""
        if rightward:
            self.update_left(site + 1)
        else:
            self.update_right(site - 1)

    def matvec(self, site, x):
        return one_site_matvec(self.left[site], self.w[site], self.right[site], x)

    def full_matrix(self, site):
        return one_site_full_matrix(self.left[site], self.w[site], self.right[site])


def expectation(mps: list[np.ndarray], mpo: list[np.ndarray]) -> float:
    """<psi|O|psi> without normalisation (MatrixProductStateMeasurements.expectation_value,
    matrix_product_state.py:447-453)."""
    from .models import uniform

    env = np.ones((1, 1, 1))
    for a, w in zip(mps, uniform(mpo)):
        env = update_left(env, a, w)
    return float(env.reshape(-1)[0])


def norm_sq(mps: list[np.ndarray]) -> float:
    env = np.ones((1, 1))
    for a in mps:
        t = np.tensordot(env, a, axes=([0], [0]))  # (a', s, c)
        env = np.tensordot(t, a, axes=([0, 1], [0, 1]))  # (c, c')
    return float(env[0, 0])


def variance(mps: list[np.ndarray], mpo: list[np.ndarray]) -> float:
    """<H^2> - <H>^2 with the MPO square, no normalisation (matrix_product_state.py:367-370)."""
    from .operators import mpo_square

    return expectation(mps, mpo_square(mpo)) - expectation(mps, mpo) ** 2


def local_sz(mps: list[np.ndarray]) -> np.ndarray:
    """<Sz_i> / <psi|psi> for every site (one-site MPO expectation, a reporting addition)."""
    n = len(mps)
    sz = np.diag([0.5, -0.5])
    # left and right norm environments
    lefts = [np.ones((1, 1))]
    for a in mps[:-1]:
        t = np.tensordot(lefts[-1], a, axes=([0], [0]))
        lefts.append(np.tensordot(t, a, axes=([0, 1], [0, 1])))
    rights = [np.ones((1, 1))]
    for a in mps[:0:-1]:
        t = np.tensordot(a, rights[-1], axes=([2], [0]))  # (a, s, c')
        rights.append(np.tensordot(t, a, axes=([1, 2], [1, 2])))
    rights = rights[::-1]
    out = np.empty(n)
    for i, a in enumerate(mps):
        t = np.tensordot(lefts[i], a, axes=([0], [0]))  # (a', s, c)
        t = np.tensordot(t, rights[i], axes=([2], [0]))  # (a', s, c')
        num = np.einsum("xsy,st,xty->", t, sz, a)
        den = np.einsum("xsy,xsy->", t, a)
        out[i] = num / den
    return out
