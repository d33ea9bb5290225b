"""Exact diagonalisation on the device (tnpy/exact_diagonalization.py:10-250).

``ExactDiagonalization(mpo)`` builds the dense Hamiltonian of the MPO on the GPU (one thread
per matrix element carrying the MPO transfer product, site 0 the most significant digit as in
FullHamiltonian) and computes its full spectrum with the one-sided Jacobi SVD of the shifted,
positive definite H + c I (eigenvalues = singular values - c, eigenvectors = singular vectors).
``evals`` is a host array in ascending order (as np.linalg.eigh returns it); ``matrix`` and
``evecs`` are FP64 device tensors (column k of ``evecs`` belongs to ``evals[k]``). The
measurements restate the reference's on the device: reduced density matrix spectra by the
Jacobi SVD of the reshaped eigenvector, local operators as Kronecker products applied with the
library's FP64 GEMM.
"""
from __future__ import annotations

import logging
from typing import Sequence

import numpy as np
import torch

from . import kernels as K
from ._lib import check, lib, ptr, stream_ptr
from .operators import MatrixProductOperator

logger = logging.getLogger("tnpy")

MAX_DIM = 4096


def full_hamiltonian(mpo: MatrixProductOperator, device=None) -> torch.Tensor:
    """Dense H[(k_0..k_{n-1}), (b_0..b_{n-1})] of the MPO on the device (operators.py:119-166);
    raises ResourceWarning above 4096 x 4096 as the reference does (:140-143)."""
    n, d = mpo.n_sites, mpo.phys_dim
    if d**n > MAX_DIM:
        raise ResourceWarning(f"Requesting more than {n} sites with physical dim {d}.")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    w = mpo.uniform()
    D = max(max(x.shape[0], x.shape[1]) for x in w)
    packed = np.zeros((n, D, D, d, d))
    for s, x in enumerate(w):
        packed[s, : x.shape[0], : x.shape[1]] = x
    wd = torch.from_numpy(packed).to(dev)
    dim = d**n
    H = torch.empty((dim, dim), dtype=torch.float64, device=dev)
    check("tnx_full_hamiltonian", lib.tnx_full_hamiltonian(ptr(wd), n, D, d, ptr(H), stream_ptr()))
    return H


def eigh_full(H: torch.Tensor):
    """All eigenpairs of a symmetric device matrix, ascending: one-sided Jacobi SVD of H + c I
    (c = max row sum |H| + 1 makes it positive definite). Returns (evals host array, evecs)."""
    dim = H.shape[0]
    A = H.clone()
    shift = torch.empty(1, dtype=torch.float64, device=H.device)
    check("tnx_shift_to_spd", lib.tnx_shift_to_spd(ptr(A), dim, ptr(shift), 0, stream_ptr()))
    u, s, _ = K.svd(A, want_u=True, want_vt=False)
    c = float(shift.item())
    evals = (s - c).flip(0).cpu().numpy()
    evecs = u.flip(1).contiguous()
    return evals, evecs


class ExactDiagonalization:
    def __init__(self, mpo: MatrixProductOperator, proj: np.ndarray | None = None, device=None):
        """Dense H of ``mpo`` (optionally P^T H P with the projector ``proj``) and its full
        spectrum, computed at construction (exact_diagonalization.py:10-60)."""
        self._mpo = mpo
        self._n_sites, self._phys_dim = mpo.n_sites, mpo.phys_dim
        H = full_hamiltonian(mpo, device)
        self._proj = proj
        if proj is not None:
            p = torch.as_tensor(np.asarray(proj, dtype=float)).to(H.device).contiguous()
            H = K.gemm(p, K.gemm(H, p), trans_a=True)
        self._matrix = H
        self._evals, self._evecs = eigh_full(H)

    @property
    def n_sites(self) -> int:
        return self._n_sites

    @property
    def phys_dim(self) -> int:
        return self._phys_dim

    @property
    def proj(self):
        return self._proj

    @property
    def matrix(self) -> torch.Tensor:
        return self._matrix

    @property
    def evals(self) -> np.ndarray:
        """Eigenvalues in ascending order."""
        return self._evals

    @property
    def evecs(self) -> torch.Tensor:
        """Eigenvectors as device columns, in the order of ``evals``."""
        return self._evecs

    def _check_level(self, level_idx: int):
        if not 0 <= level_idx < len(self._evals):
            raise ValueError("Parameter `level_idx` has to be lower than truncation dimension.")

    def reduced_density_matrix(self, site: int, level_idx: int = 0) -> np.ndarray:
        """Squared Schmidt values of eigenvector ``level_idx`` across the bond site | site+1
        (exact_diagonalization.py:62-90), from the Jacobi SVD of the reshaped vector."""
        if not 0 <= site < self.n_sites - 1:
            raise ValueError("Parameter `site` for bi-partition has to be within the system size.")
        self._check_level(level_idx)
        d, n = self.phys_dim, self.n_sites
        shape = (d ** (site + 1), -1) if site < n // 2 else (-1, d ** (n - site - 1))
        m = self._evecs[:, level_idx].contiguous().reshape(shape)
        if m.shape[0] < m.shape[1]:
            m = m.T
        _, s, _ = K.svd(m.contiguous(), want_u=False, want_vt=False)
        return (s * s).cpu().numpy()

    def entanglement_entropy(self, site: int, level_idx: int = 0, nan_to_num: bool = False) -> float:
        """-rho . log(rho) of the reduced density matrix spectrum (:92-109)."""
        rho = self.reduced_density_matrix(site, level_idx)
        with np.errstate(divide="ignore", invalid="ignore"):
            entropy = -1 * rho @ np.log(rho)
        return float(np.nan_to_num(entropy)) if nan_to_num else float(entropy)

    @staticmethod
    def kron_operators(operators: Sequence[np.ndarray]) -> np.ndarray:
        """Kronecker product of a sequence of operators (:111-128)."""
        opt = operators[0]
        for next_opt in operators[1:]:
            opt = np.kron(opt, next_opt)
        return opt

    def _sandwich(self, op: np.ndarray, level_idx: int) -> float:
        v = self._evecs[:, level_idx].contiguous().reshape(-1, 1)
        o = torch.as_tensor(np.asarray(op, dtype=float)).to(v.device).contiguous()
        return float(K.gemm(v, K.gemm(o, v), trans_a=True).item())

    def one_point_function(self, operator: np.ndarray, site: int, level_idx: int = 0) -> float:
        """<psi_l| O_site |psi_l> (:130-152)."""
        d = self.phys_dim
        if operator.shape != (d, d):
            raise ValueError(f"Operator shape mismatched with physical dims {d}.")
        self._check_level(level_idx)
        op = self.kron_operators([np.eye(d**site), operator, np.eye(d ** (self.n_sites - site - 1))])
        return self._sandwich(op, level_idx)

    def two_point_function(self, operator1: np.ndarray, operator2: np.ndarray, site1: int, site2: int,
                           level_idx: int) -> float:
        """<psi_l| O1_site1 O2_site2 |psi_l> (:154-197)."""
        d = self.phys_dim
        if operator1.shape != (d, d) or operator2.shape != (d, d):
            raise ValueError(f"Operator shape mismatched with physical dims {d}.")
        if site1 == site2:
            raise ValueError("Two sites must not be the same site.")
        self._check_level(level_idx)
        site1, site2 = sorted((site1, site2))
        op = self.kron_operators([np.eye(d**site1), operator1, np.eye(d ** (abs(site1 - site2) - 1)), operator2,
                                  np.eye(d ** (self.n_sites - site2 - 1))])
        return self._sandwich(op, level_idx)

    def connected_two_point_function(self, operator1, operator2, site1: int, site2: int, level_idx: int) -> float:
        """:199-223."""
        return self.two_point_function(operator1, operator2, site1, site2, level_idx) - \
            self.one_point_function(operator1, site1, level_idx) * self.one_point_function(operator2, site2, level_idx)

    def variance(self, operator=None, tol: float = 1e-12) -> np.ndarray:
        """diag(V^T O^2 V - (V^T O V)^2) over all eigenvectors V (:225-250); default O = H."""
        o = self._matrix if operator is None else \
            torch.as_tensor(np.asarray(operator, dtype=float)).to(self._matrix.device).contiguous()
        V = self._evecs
        ov = K.gemm(o, V)
        first = K.gemm(V, ov, trans_a=True)
        second = K.gemm(ov, ov, trans_a=True)  # V^T O^2 V = (O V)^T (O V), O symmetric
        var = (second - first * first).cpu().numpy()
        if not np.allclose(np.zeros(var.shape), var - np.diagflat(np.diag(var)), atol=tol):
            logger.warning("Expectation value may contain large off-diagonal elements.")
        return np.diag(var).copy()
