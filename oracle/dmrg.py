"""One-site finite DMRG (oracle), restating tnpy/finite_dmrg.py:32-263.

* eigensolver dispatch (finite_dmrg.py:97-111): dense ``np.linalg.eigh`` of the
  effective Hamiltonian when the site tensor has fewer than
  ``exact_solver_dim`` (200) elements, otherwise a matrix-free Lanczos
  (``scipy.sparse.linalg.eigsh``, which='SA', restating ``primme.eigsh`` of
  linalg.py:64-87) started from the current site tensor;
* perturbation psi += 1e-5 H_eff psi without renormalisation (:116-141);
* SVD gauge move without truncation, S V^T pushed unnormalised (mps.py:187-225);
* sweeps alternate rightward (sites 0..n-2) / leftward (n-1..1) starting
  rightward (:241-243); stop when |dE| < tol or after max_sweep (:173-212).
"""
from __future__ import annotations

import time

import numpy as np
import scipy.sparse.linalg as spla

from . import mps as M


def eigsh_lowest(op, v0: np.ndarray, tol: float):
    """Lowest eigenpair of a symmetric operator (linalg.py:64-87, which='SA', k=1)."""
    n = v0.size
    lin = spla.LinearOperator((n, n), matvec=op, dtype=float)
    vals, vecs = spla.eigsh(lin, k=1, which="SA", v0=v0.reshape(-1), tol=tol, ncv=min(n, 24))
    return float(vals[0]), vecs[:, 0]


class FiniteDMRG:
    def __init__(self, mpo, chi: int, mps=None, exact_solver_dim: int = 200, seed: int = 1234,
                 eig_tol: float = 1e-12):
        n = len(mpo)
        d = mpo[0].shape[-1]
        self.mpo = mpo
        self.chi = chi
        self.exact_solver_dim = exact_solver_dim
        self.eig_tol = eig_tol
        self.mps = [a.copy() for a in mps] if mps is not None else M.random_mps(n, chi, d, seed)
        self.env = M.Environment(mpo, self.mps)
        self.energies = [np.nan]
        self.variances = [np.nan]
        self.sweep_seconds: list[float] = []
        self.n = n

    def one_site_solver(self, site: int, tol: float):
        x0 = self.mps[site]
        if x0.size < self.exact_solver_dim:
            evals, evecs = np.linalg.eigh(self.env.full_matrix(site))
            return float(evals[0]), evecs[:, 0].reshape(x0.shape)
        e, v = eigsh_lowest(
            lambda v: self.env.matvec(site, v.reshape(x0.shape)).reshape(-1), x0, self.eig_tol
        )
        return e, v.reshape(x0.shape)

    def perturb(self, site: int, alpha: float = 1e-5):
        psi = self.mps[site]
        self.mps[site] = psi + alpha * self.env.matvec(site, psi)

    def sweep(self, rightward: bool, tol: float):
        sites = range(self.n - 1) if rightward else range(self.n - 1, 0, -1)
        energy = None
        for site in sites:
            energy, psi = self.one_site_solver(site, tol)
            self.mps[site] = psi
            self.perturb(site)
            M.split_tensor(self.mps, site, rightward)
            self.env.update(site, rightward)
        return energy

    def run(self, tol: float = 1e-8, max_sweep: int = 100, with_variance: bool = True):
        for n_sweep in range(1, max_sweep + 1):
            rightward = n_sweep % 2 == 1
            t0 = time.perf_counter()
            e = self.sweep(rightward, tol)
            self.sweep_seconds.append(time.perf_counter() - t0)
            self.energies.append(e)
            self.variances.append(M.variance(self.mps, self.mpo) if with_variance else np.nan)
            if abs(self.energies[-1] - self.energies[-2]) < tol:
                break
        return self.energies[1:]


class ShiftInvertDMRG(FiniteDMRG):
    """Shift-invert one-site DMRG (restating tnpy/finite_dmrg.py:266-407).

    The MPO is that of H - eps; each site solves the generalised problem
    (H - eps) phi = lambda (H - eps)^2 phi for the smallest lambda, with the second operator from
    the environments of the MPO square: scipy.linalg.eigh(a, b) of the dense one-site operators
    (:349-356 below exact_solver_dim elements; primme.eigsh(A, M=B) above it, :357-363, whose
    converged pair is the same: ARPACK cannot stand in for it, its inversion of the
    ill-conditioned (H - eps)^2 by GMRES fails, so the restatement is dense at every size and
    meant for chains of a few tens of sites). Energies are reported as 1/lambda + offset
    (:386-395) and the state restored as psi = (H - eps) phi, site by site (:314-343)."""

    def __init__(self, mpo, chi: int, offset: float = 0.0, mps=None, exact_solver_dim: int = 200, seed: int = 1234,
                 eig_tol: float = 1e-12):
        super().__init__(mpo, chi, mps=mps, exact_solver_dim=exact_solver_dim, seed=seed, eig_tol=eig_tol)
        from .operators import mpo_square

        self.env2 = M.Environment(mpo_square(mpo), self.mps)
        self.offset = offset
        self.restored = None

    def one_site_solver(self, site: int, tol: float):
        import scipy.linalg as spl

        x0 = self.mps[site]
        a, b = self.env.full_matrix(site), self.env2.full_matrix(site)
        w, v = spl.eigh(0.5 * (a + a.T), b=0.5 * (b + b.T), subset_by_index=[0, 0])
        return float(w[0]), v[:, 0].reshape(x0.shape)

    def sweep(self, rightward: bool, tol: float):
        sites = range(self.n - 1) if rightward else range(self.n - 1, 0, -1)
        energy = None
        for site in sites:
            energy, psi = self.one_site_solver(site, tol)
            self.mps[site] = psi
            self.perturb(site)
            M.split_tensor(self.mps, site, rightward)
            self.env.update(site, rightward)
            self.env2.update(site, rightward)
        return energy

    def run(self, tol: float = 1e-7, max_sweep: int = 100, with_variance: bool = False):
        energies = super().run(tol, max_sweep, with_variance=False)
        self.restored = restore_mps(self.mps, self.mpo)
        return (np.reciprocal(energies) + self.offset).tolist()


def restore_mps(mps, mpo):
    """psi = (H - eps) phi as an MPS: site tensor A'[(a w), k, (c v)] = sum_b W[w, v, k, b] A[a, b, c]
    (tnpy/finite_dmrg.py:314-343)."""
    from .models import uniform

    out = []
    for a, w in zip(mps, uniform(mpo)):
        t = np.einsum("wvkb,abc->awkcv", w, a)
        al, wl, d, cr, vr = t.shape
        out.append(t.reshape(al * wl, d, cr * vr))
    return out
