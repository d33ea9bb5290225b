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
