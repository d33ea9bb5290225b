"""Measurements on a tSDRG tree of isometries (tnpy/tsdrg.py:711-1028), on the device.

The tree's root carries k renormalised eigenstates |psi_l> (l = level_idx). Everything that is
an operator sandwich <psi_i| O |psi_j> is computed the way tSDRG builds its effective
Hamiltonian: the MPO of O is renormalised up the tree, node by node in merge order, with the
batched spectrum projector W' = V^T (W_left W_right) V (tnx_tsdrg_project), so that the root
holds the k x k matrix of O between the kept states. Local operators become product MPOs of
bond 1 (the reference contracts the same numbers along the paths of the sites involved).
The reduced density matrix of a bipartition is built from the state vector of |psi_l>,
expanded top-down through the isometries with FP64 GEMMs of the library (2^n amplitudes;
chains up to 24 sites), on the smaller side as the reference does.
"""
from __future__ import annotations

import logging

import numpy as np
import torch

from . import kernels as K
from .operators import MatrixProductOperator

logger = logging.getLogger("tnpy")

MAX_STATE_SITES = 24


def _local_mpo(n: int, d: int, ops: dict, dev) -> list[torch.Tensor]:
    """Product MPO of bond dimension 1: ops[site] on the listed sites, identity elsewhere."""
    out = []
    for s in range(n):
        m = np.asarray(ops.get(s, np.eye(d)), dtype=float)
        if m.shape != (d, d):
            raise ValueError(f"Operator shape mismatched with physical dims {d}.")
        out.append(torch.from_numpy(m.reshape(1, 1, d, d).copy()).to(dev))
    return out


class TreeTensorNetworkMeasurements:
    def __init__(self, tree, phys_dim: int = 2, device=None):
        """Measurements of the states held by ``tree`` (tsdrg.py:711-720); the tree comes from a
        finished TreeTensorNetworkSDRG run (its internal nodes hold the isometries), phys_dim is
        the leaves' physical dimension."""
        tree._check_root()
        self._tree = tree
        self._d = int(phys_dim)
        self._dev = tree.root.data.device if device is None else torch.device(device)

    @property
    def tree(self):
        return self._tree

    @property
    def n_levels(self) -> int:
        return int(self._tree.root.data.shape[2])

    # ---- sandwiches ----------------------------------------------------------------------
    def _renormalise(self, site_tensors: list[torch.Tensor]) -> torch.Tensor:
        """Root k x k matrix of the MPO given by its (dl, dr, d, d) site tensors."""
        from .tsdrg import project

        tree = self._tree
        n = tree.n_leaves
        cache = {s: site_tensors[s].contiguous() for s in range(n)}
        for node_id in range(n, tree.n_nodes):
            node = tree[node_id]
            v = node.data
            m1, m2, k = v.shape
            (w,) = project([(cache[node.left.node_id], cache[node.right.node_id], v.reshape(m1 * m2, k))], self._dev)
            cache[node_id] = w
            del cache[node.left.node_id], cache[node.right.node_id]
        root = cache[tree.root_id]
        return root.reshape(root.shape[2], root.shape[3])

    def sandwich(self, mpo: MatrixProductOperator | None = None) -> torch.Tensor:
        """<psi_i| O |psi_j> for the MPO O, or <psi_i|psi_j> without one (tsdrg.py:765-784),
        as a k x k device tensor."""
        n = self._tree.n_leaves
        if mpo is None:
            return self._renormalise(_local_mpo(n, self._d, {}, self._dev))
        if mpo.n_sites != n:
            raise ValueError(f"MPO has {mpo.n_sites} sites, the tree {n}")
        return self._renormalise(mpo.device_tensors(self._dev))

    def expectation_value(self, mpo: MatrixProductOperator, tol: float = 1e-12) -> np.ndarray:
        """diag <psi_l| O |psi_l> (tsdrg.py:786-806); warns when an off-diagonal element exceeds tol."""
        m = self.sandwich(mpo).cpu().numpy()
        if not np.allclose(np.zeros(m.shape), m - np.diagflat(np.diag(m)), atol=tol):
            logger.warning("Expectation value may contain large off-diagonal elements.")
        return np.diag(m).copy()

    def variance(self, mpo: MatrixProductOperator) -> np.ndarray:
        """<O^2> - <O>^2 per level with the MPO square (tsdrg.py:1005-1016)."""
        return self.expectation_value(mpo.square()) - self.expectation_value(mpo) ** 2

    def _check_level(self, level_idx: int):
        if not 0 <= level_idx < self.n_levels:
            raise ValueError("Parameter `level_idx` has to be lower than truncation dimension.")

    def one_point_function(self, operator, site: int, level_idx: int) -> float:
        """<psi_l| O_site |psi_l> (tsdrg.py:899-932)."""
        self._check_level(level_idx)
        n = self._tree.n_leaves
        m = self._renormalise(_local_mpo(n, self._d, {site: operator}, self._dev))
        return float(m[level_idx, level_idx].item())

    def two_point_function(self, operator1, operator2, site1: int, site2: int, level_idx: int) -> float:
        """<psi_l| O1_site1 O2_site2 |psi_l> (tsdrg.py:934-980)."""
        if site1 == site2:
            raise ValueError("Two sites must not be the same site.")
        self._check_level(level_idx)
        n = self._tree.n_leaves
        m = self._renormalise(_local_mpo(n, self._d, {site1: operator1, site2: operator2}, self._dev))
        return float(m[level_idx, level_idx].item())

    def connected_two_point_function(self, operator1, operator2, site1: int, site2: int, level_idx: int) -> float:
        """tsdrg.py:982-1003."""
        return self.two_point_function(operator1, operator2, site1, site2, level_idx) - \
            self.one_point_function(operator1, site1, level_idx) * self.one_point_function(operator2, site2, level_idx)

    # ---- bipartitions ----------------------------------------------------------------------
    def state_vector(self, level_idx: int) -> torch.Tensor:
        """Amplitudes of |psi_l> over the 2^n product basis (site 0 the most significant digit, as
        FullHamiltonian orders it), expanded top-down: the root isometry's column l, then every
        node's bond replaced by its children's bonds with one FP64 GEMM (V (m1 m2 x k) times the
        amplitudes with that bond moved to the front)."""
        self._check_level(level_idx)
        tree = self._tree
        n = tree.n_leaves
        if n > MAX_STATE_SITES:
            raise ValueError(f"state vectors are formed for chains up to {MAX_STATE_SITES} sites (got {n})")
        root = tree.root
        m1, m2, _ = root.data.shape
        psi = root.data[:, :, level_idx].contiguous().reshape(m1 * m2)
        blocks = [root.left, root.right]  # current factorisation, left to right
        dims = [m1, m2]
        while any(not b.is_leaf for b in blocks):
            j = next(i for i, b in enumerate(blocks) if not b.is_leaf)
            node = blocks[j]
            a, b_, k = node.data.shape
            pre = int(np.prod(dims[:j])) if j else 1
            post = int(np.prod(dims[j + 1:])) if j + 1 < len(dims) else 1
            t = psi.reshape(pre, k, post).permute(1, 0, 2).contiguous().reshape(k, pre * post)
            u = K.gemm(node.data.reshape(a * b_, k).contiguous(), t)  # (a b, pre post)
            psi = u.reshape(a, b_, pre, post).permute(2, 0, 1, 3).contiguous().reshape(-1)
            blocks[j:j + 1] = [node.left, node.right]
            dims[j:j + 1] = [a, b_]
        return psi

    def reduced_density_matrix(self, site: int, level_idx: int) -> np.ndarray:
        """Reduced density matrix of |psi_l> for the cut between site and site+1, on the smaller
        side (tsdrg.py:841-883); dense, 2^|side| x 2^|side|."""
        n = self._tree.n_leaves
        if not 0 <= site < n - 1:
            raise ValueError("Parameter `site` for bi-partition has to be within the system size.")
        self._check_level(level_idx)
        d = self._d
        psi = self.state_vector(level_idx).reshape(d ** (site + 1), -1)
        left_smaller = (site + 1) / (n - site) < 1
        rho = K.gemm(psi, psi, trans_b=True) if left_smaller else K.gemm(psi, psi, trans_a=True)
        return rho.cpu().numpy()

    def entanglement_entropy(self, site: int, level_idx: int, nan_to_num: bool = False) -> float:
        """von Neumann entropy -sum rho log rho of the cut (tsdrg.py:885-897); the spectrum of the
        reduced density matrix from the device Jacobi eigensolver."""
        from . import linalg

        rdm = self.reduced_density_matrix(site, level_idx)
        w, _ = linalg.eigh(rdm, k=rdm.shape[0])
        rho = w.cpu().numpy()[::-1]
        with np.errstate(divide="ignore", invalid="ignore"):
            entropy = -1 * rho @ np.log(rho)
        return float(np.nan_to_num(entropy)) if nan_to_num else float(entropy)

    def wave_func_coeff(self, level_idx: int):
        return NotImplemented

    def squared_moduli(self, level_idx: int):
        return NotImplemented

    def kullback_leibler_divergence(self):
        return NotImplemented

    def participation_entropy(self):
        return NotImplemented
