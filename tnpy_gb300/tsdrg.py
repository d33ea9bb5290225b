"""Tree-tensor-network SDRG on the GPU (tnpy/tsdrg.py:18-709).

``TreeTensorNetworkSDRG(mpo, chi).run()`` (alias ``TSDRG``) keeps the reference's greedy
procedure (:671-696): solve every two-block Hamiltonian, merge the bond with the largest
truncation gap, renormalise the merged MPO tensor with the kept eigenvectors, re-solve the
one or two neighbouring bonds, until one tensor is left. ``BatchedTSDRG`` runs many
independent chains (disorder realisations) in lockstep so that every step is one batched
launch of each kernel: block-Hamiltonian assembly, the batched eigensolver and the
spectrum projector.

Host work is bookkeeping only: the argmax over gaps (one small device->host copy per step)
and the binary tree of node ids.
"""
from __future__ import annotations

import logging
from typing import Dict, List, Sequence

import numpy as np
import torch

from . import kernels as K
from ._lib import check, lib, ptr, stream_ptr
from .operators import MatrixProductOperator

logger = logging.getLogger("tnpy")


# ------------------------------------------------------------------ tree bookkeeping
class Node:
    """Binary-tree node holding an isometry (tsdrg.py:18-61); leaves hold the MPO tensors."""

    def __init__(self, node_id: int, left: "Node | None" = None, right: "Node | None" = None, data=None):
        self._node_id = node_id
        self._left = left
        self._right = right
        self.data = data

    def __repr__(self):
        lid = None if self.left is None else self.left.node_id
        rid = None if self.right is None else self.right.node_id
        shape = None if self.data is None else tuple(self.data.shape)
        return f"Node(id={self.node_id}, left_id={lid}, right_id={rid}, shape={shape})"

    @property
    def node_id(self) -> int:
        return self._node_id

    @property
    def left(self):
        return self._left

    @property
    def right(self):
        return self._right

    @property
    def is_leaf(self) -> bool:
        return self.left is None and self.right is None


class TensorTree:
    """Bottom-up binary tree of tSDRG isometries (tsdrg.py:64-441, without plotting)."""

    def __init__(self, mpo_or_n):
        n = mpo_or_n if isinstance(mpo_or_n, int) else mpo_or_n.n_sites
        leaves = [None] * n if isinstance(mpo_or_n, int) else list(mpo_or_n)
        self._root_id: int | None = None
        self._tree: Dict[int, Node] = {s: Node(s, data=leaves[s]) for s in range(n)}
        self._n_leaves = n
        self._horizon = list(range(n))

    def __iter__(self):
        return iter(self._tree.values())

    def __getitem__(self, node_id: int) -> Node:
        return self._tree[node_id]

    def __setitem__(self, node_id: int, node: Node):
        self._tree[node_id] = node

    @property
    def root_id(self):
        return self._root_id

    @property
    def root(self) -> Node:
        if self._root_id is None:
            raise KeyError("Can't find root in tree.")
        return self[self._root_id]

    @property
    def leaves(self) -> Dict[int, Node]:
        return {k: self._tree[k] for k in range(self._n_leaves)}

    @property
    def horizon(self) -> List[int]:
        return self._horizon

    @property
    def n_nodes(self) -> int:
        return len(self._tree)

    @property
    def n_leaves(self) -> int:
        return self._n_leaves

    def fuse(self, left_id: int, right_id: int, new_id: int, data):
        """tsdrg.py:163-219."""
        if self.root_id is not None:
            raise RuntimeError("Can't perform fuse on a grown tree.")
        self[new_id] = Node(new_id, left=self[left_id], right=self[right_id], data=data)
        self._horizon[self._horizon.index(left_id)] = new_id
        self._horizon.remove(right_id)
        if self.n_nodes == 2 * self.n_leaves - 1:
            self._root_id = new_id

    def _check_root(self):
        if self._root_id is None:
            raise KeyError("Can't find root in tree.")

    @property
    def n_layers(self) -> int:
        self._check_root()

        def depth(node):
            return 0 if node is None else max(depth(node.left), depth(node.right)) + 1

        return depth(self.root)

    def find_path(self, node_id: int, return_itself: bool = False) -> List[int]:
        """tsdrg.py:317-358."""
        self._check_root()
        path: List[int] = []

        def find(node) -> bool:
            if node is None:
                return False
            path.append(node.node_id)
            if node.node_id == node_id or find(node.left) or find(node.right):
                return True
            path.pop()
            return False

        if not find(self.root):
            raise KeyError("The given node_id is not found in tree.")
        return path if return_itself else path[:-1]

    def common_ancestor(self, node_id1: int, node_id2: int, lowest: bool = False):
        """tsdrg.py:360-384."""
        p1 = self.find_path(node_id1, return_itself=True)
        p2 = self.find_path(node_id2, return_itself=True)
        common = []
        for x, y in zip(p1, p2):
            if x != y:
                break
            common.append(x)
        else:
            common = p1[:-1] if p1 == p2 else common
        return common[-1] if lowest else common


# ------------------------------------------------------------------ device helpers
def _ptr_array(tensors: Sequence[torch.Tensor], dev) -> torch.Tensor:
    return torch.tensor([t.data_ptr() for t in tensors], dtype=torch.int64, device=dev)


def block_hamiltonians(pairs, dev) -> tuple[list[torch.Tensor], list[int]]:
    """Two-block Hamiltonians of (W1, W2) pairs, one launch (tsdrg.py:607-631)."""
    if not pairs:
        return [], []
    D = pairs[0][0].shape[1]
    sizes = [w1.shape[2] * w2.shape[2] for w1, w2 in pairs]
    offs = np.concatenate([[0], np.cumsum([s * s for s in sizes])[:-1]]).astype(np.int64)
    packed = torch.empty(int(sum(s * s for s in sizes)), dtype=torch.float64, device=dev)
    meta = torch.tensor([[w1.shape[2], w2.shape[2], w1.shape[0], w2.shape[1]] for w1, w2 in pairs],
                        dtype=torch.int32, device=dev).reshape(-1)
    p1 = _ptr_array([w1 for w1, _ in pairs], dev)
    p2 = _ptr_array([w2 for _, w2 in pairs], dev)
    off_t = torch.from_numpy(offs).to(dev)
    check("tnx_tsdrg_block_hamiltonian",
          lib.tnx_tsdrg_block_hamiltonian(ptr(p1), ptr(p2), ptr(meta), int(D), ptr(packed), ptr(off_t), len(pairs),
                                          int(max(sizes)), stream_ptr()))
    mats = [packed[int(o): int(o) + s * s].view(s, s) for o, s in zip(offs, sizes)]
    return mats, sizes


KRON_MAX_NODE = 32
KRON_MAX_P = 48


def kron_eigh(pairs, chi: int, dev, precision: str = "mixed"):
    """Lowest min(chi, m) eigenpairs of the two-block Hamiltonians of (W1, W2) pairs without
    forming them (Kronecker-sum Chebyshev subspace iteration + FP64 Rayleigh-Ritz, one CTA per
    block). Returns (evals [batch, keep] device, evecs [batch, max_m, keep] device, ks, iters), iters
    negative for blocks whose subspace iteration did not converge."""
    D = pairs[0][0].shape[1]
    ms = [(w1.shape[2], w2.shape[2]) for w1, w2 in pairs]
    ks = [min(chi, a * b) for a, b in ms]
    # guard vectors: the k-th wanted pair converges at a rate set by the gap to the (p+1)-th
    ps = [min(a * b, k + max(16, k // 2), KRON_MAX_P) for (a, b), k in zip(ms, ks)]
    keep = max(ks)
    max_m = max(a * b for a, b in ms)
    meta = torch.tensor([[a, b, w2.shape[1], k, p] for (a, b), k, p, (_, w2) in zip(ms, ks, ps, pairs)],
                        dtype=torch.int32, device=dev).reshape(-1)
    p1 = _ptr_array([w1 for w1, _ in pairs], dev)
    p2 = _ptr_array([w2 for _, w2 in pairs], dev)
    evals = torch.full((len(pairs), keep), float("nan"), dtype=torch.float64, device=dev)
    evecs = torch.zeros((len(pairs), max_m, keep), dtype=torch.float64, device=dev)
    iters = torch.zeros(len(pairs), dtype=torch.int32, device=dev)
    code = K.precision_code(precision)
    nbytes = lib.tnx_tsdrg_block_eigh_workspace_bytes(len(pairs), max_m, keep, code)
    wp, wn = K.Workspace.get(nbytes, dev)
    check("tnx_tsdrg_block_eigh", lib.tnx_tsdrg_block_eigh(ptr(p1), ptr(p2), ptr(meta), int(D), len(pairs), max_m,
                                                         keep, code, ptr(evals), ptr(evecs), ptr(iters), wp, wn,
                                                         stream_ptr()))
    del p1, p2, meta
    return evals, evecs, ks, iters


def project(pairs_v, dev) -> list[torch.Tensor]:
    """Renormalised MPO tensors W' = V^T (W1 W2) V for (W1, W2, V) triples (tsdrg.py:633-669)."""
    if not pairs_v:
        return []
    D = pairs_v[0][0].shape[1]
    small = all(w1.shape[2] <= 32 and w2.shape[2] <= 32 and v.shape[1] <= 32 for w1, w2, v in pairs_v)
    outs = [torch.empty((w1.shape[0], w2.shape[1], v.shape[1], v.shape[1]), dtype=torch.float64, device=dev)
            for w1, w2, v in pairs_v]
    if small:
        vs = [v.contiguous() for _, _, v in pairs_v]
        if vs:
            meta = torch.tensor([[w1.shape[2], w2.shape[2], w1.shape[0], w2.shape[1], v.shape[1]]
                                 for (w1, w2, _), v in zip(pairs_v, vs)], dtype=torch.int32, device=dev).reshape(-1)
            # the pointer arrays must stay referenced until the launch is queued: a freed
            # temporary could be handed to the next allocation of the same call
            p1 = _ptr_array([p[0] for p in pairs_v], dev)
            p2 = _ptr_array([p[1] for p in pairs_v], dev)
            pv = _ptr_array(vs, dev)
            po = _ptr_array(outs, dev)
            check("tnx_tsdrg_project", lib.tnx_tsdrg_project(
                ptr(p1), ptr(p2), ptr(pv), ptr(meta), int(D), ptr(po), len(pairs_v),
                max(p[0].shape[2] for p in pairs_v), max(p[1].shape[2] for p in pairs_v), max(v.shape[1] for v in vs),
                stream_ptr()))
            del p1, p2, pv, po
            return outs
    # general sizes: M_lr = sum_w W1[l,w] (x) W2[w,r] by the block-Hamiltonian kernel, then two GEMMs
    for (w1, w2, v), out in zip(pairs_v, outs):
        dl1, dr2 = w1.shape[0], w2.shape[1]
        for l in range(dl1):
            for r in range(dr2):
                w1l = w1[l:l + 1].contiguous()
                # select column r of W2 by a copy whose last column is W2[:, r]
                w2r = w2[:, r:r + 1].contiguous()
                (m,), _ = block_hamiltonians([(w1l, w2r)], dev)
                out[l, r] = K.gemm(v, K.gemm(m, v), trans_a=True)
    return outs


# ------------------------------------------------------------------ the algorithm
class _Chain:
    """State of one realisation: coarse-grained MPO cache, horizon, gaps, kept vectors."""

    def __init__(self, mpo: MatrixProductOperator, chi: int, dev, precision: str = "fp64", mode: str = "lowest",
                 offset: float = 0.0):
        self.n = mpo.n_sites
        self.chi = chi
        self.precision = precision
        self.mode = mode  # which block eigenpairs are kept: lowest, highest, shift_invert
        self.offset = offset
        self.cache = [w.contiguous() for w in mpo.device_tensors(dev)]
        self.tree = TensorTree(self.n)
        self.gap: list[float] = []
        self.evecs: list[torch.Tensor] = []
        self.evals = None
        self.step = 0
        self.done = False


def _gap(evals: np.ndarray, chi: int, mode: str = "lowest") -> float:
    """truncation_gap (tsdrg.py:594-605), applied to the already truncated spectrum; the
    high-energy variant's gap (tsdrg.py:1054-1067) for mode 'highest'."""
    gaps = np.diff(evals)
    if mode == "highest":
        return float(gaps[-chi] if gaps.size > chi else gaps[0])
    return float(gaps[chi - 1] if gaps.size > chi else gaps[-1])


def _select(c: "_Chain", ev: np.ndarray, vec: torch.Tensor):
    """Kept pairs of a fully solved block for the variants: the chi highest (tsdrg.py:1044-1052),
    or shift-invert (tsdrg.py:1078-1089): eigh(H, H^2) has eigenvalues 1/E with unit vectors
    H x = sign(E) v, so the chi pairs of smallest 1/E are kept and reported as E + offset,
    ascending."""
    m = ev.size
    if c.mode == "highest":
        k = min(m, c.chi)
        return ev[m - k:].copy(), vec[:, m - k:].contiguous()
    with np.errstate(divide="ignore"):
        lam = np.reciprocal(ev)
    order = np.argsort(lam, kind="stable")[: min(m, c.chi)]
    e_k = ev[order] + c.offset
    idx = np.argsort(e_k, kind="stable")
    sel = order[idx]
    sign = torch.from_numpy(np.sign(ev[sel])).to(vec.device)
    return e_k[idx].copy(), (vec[:, torch.from_numpy(sel).to(vec.device)] * sign[None, :]).contiguous()


# Dense block eigensolver: the FP64 Jacobi in every precision mode. The double-FP32 Jacobi
# ('df64', 2.1x faster per 64-state block) changes, on SU(2)-symmetric chains (h = 0), which
# members of degenerate multiplets are kept; on the n=128, chi=32 bench chains the resulting
# trees merge more 32 x 32 blocks, whose Kronecker solves cost more than the Jacobi saves
# (44.6 against 90 realisations/s), so it is not the default.
_dense_precision = "fp64"


def _dense(idx, chains_bonds, out, dev):
    """Dense Jacobi solve of the listed blocks (block_hamiltonian + eigh, tsdrg.py:569-631); the
    variants' blocks are solved in full and their kept pairs selected by _select."""
    pairs = [(chains_bonds[i][0].cache[chains_bonds[i][1]], chains_bonds[i][0].cache[chains_bonds[i][1] + 1])
             for i in idx]
    mats, sizes = block_hamiltonians(pairs, dev)
    full = any(chains_bonds[i][0].mode != "lowest" for i in idx)
    chi = max(chains_bonds[i][0].chi for i in idx)
    keep = max(sizes) if full else min(chi, max(sizes))
    evals, evecs = K.eigh_batched(mats, keep=keep, precision=_dense_precision)
    ev_h = evals.cpu().numpy()
    for j, (i, m) in enumerate(zip(idx, sizes)):
        c = chains_bonds[i][0]
        if c.mode != "lowest":  # the variants: every pair of the block, then their selection
            out[i] = _select(c, ev_h[j, :m].copy(), evecs[j, :m, :m])
            continue
        kept = min(m, c.chi)
        out[i] = (ev_h[j, :kept].copy(), evecs[j, :m, :kept].contiguous())


def _solve(chains_bonds, dev):
    """Solve the listed (chain, bond) blocks; returns per item (host evals, device evecs [m, kept]).

    Blocks of at most 64 states (or with nodes beyond the Kronecker kernel's limits) are formed
    densely and diagonalised by the batched Jacobi kernel; larger blocks go to the Kronecker
    subspace eigensolver in the chain's precision. Each group is one launch."""
    out = [None] * len(chains_bonds)
    dense, kron = [], []
    for i, (c, b) in enumerate(chains_bonds):
        w1, w2 = c.cache[b], c.cache[b + 1]
        m = w1.shape[2] * w2.shape[2]
        if (c.mode == "lowest" and m > 64 and w1.shape[2] <= KRON_MAX_NODE and w2.shape[2] <= KRON_MAX_NODE
                and c.chi <= 32 and w1.shape[1] <= 6):
            kron.append(i)
        else:
            dense.append(i)
    if dense:
        _dense(dense, chains_bonds, out, dev)
    if kron:
        groups: dict = {}
        for i in kron:
            groups.setdefault(chains_bonds[i][0].precision, []).append(i)
        for prec, idx in groups.items():
            pairs = [(chains_bonds[i][0].cache[chains_bonds[i][1]], chains_bonds[i][0].cache[chains_bonds[i][1] + 1])
                     for i in idx]
            chi = max(chains_bonds[i][0].chi for i in idx)
            evals, evecs, ks, iters = kron_eigh(pairs, chi, dev, precision=prec)
            ev_h = evals.cpu().numpy()
            failed = []
            for j, (i, it) in enumerate(zip(idx, iters.cpu().numpy())):
                m = pairs[j][0].shape[2] * pairs[j][1].shape[2]
                kept = min(m, chains_bonds[i][0].chi)
                out[i] = (ev_h[j, :kept].copy(), evecs[j, :m, :kept].contiguous())
                if it < 0:
                    failed.append(i)
            if failed:
                # the subspace iteration stalled (tightly clustered spectrum): exact dense solve
                logger.debug(f"tSDRG: {len(failed)} of {len(idx)} Kronecker blocks re-solved densely")
                _dense(failed, chains_bonds, out, dev)
    return out


def run_chains(chains: List[_Chain], dev):
    """Lockstep greedy merging of many chains (tsdrg.py:456-498, :671-696)."""
    init = [(c, b) for c in chains for b in range(c.n - 1)]
    res = _solve(init, dev)
    i = 0
    for c in chains:
        for _ in range(c.n - 1):
            ev, vec = res[i]
            i += 1
            c.evecs.append(vec)
            c.gap.append(_gap(ev, c.chi, c.mode))
            c.evals = ev if c.n == 2 else None
    while True:
        active = [c for c in chains if not c.done]
        if not active:
            break
        merges = []
        for c in active:
            b = int(np.argmax(np.array(c.gap)))
            merges.append((c, b))
        news = project([(c.cache[b], c.cache[b + 1], c.evecs[b]) for c, b in merges], dev)
        resolve = []
        for (c, b), w_new in zip(merges, news):
            c.step += 1
            new_id = c.n + c.step - 1
            left, right = c.tree.horizon[b], c.tree.horizon[b + 1]
            m1, m2 = c.cache[b].shape[2], c.cache[b + 1].shape[2]
            c.tree.fuse(left, right, new_id, data=c.evecs[b].reshape(m1, m2, -1))
            c.cache.pop(b + 1)
            c.cache[b] = w_new
            if len(c.cache) == 1:
                c.done = True
                continue
            c.gap.pop(b)
            c.evecs.pop(b)
            last = len(c.cache) - 1
            nb = [b] if b == 0 else ([b - 1] if b == last else [b - 1, b])
            resolve.extend((c, bond) for bond in nb)
        if resolve:
            res = _solve(resolve, dev)
            for (c, bond), (ev, vec) in zip(resolve, res):
                c.gap[bond] = _gap(ev, c.chi, c.mode)
                c.evecs[bond] = vec
                c.evals = ev
    return chains


class TreeTensorNetworkSDRG:
    def __init__(self, mpo: MatrixProductOperator, chi: int, device=None, precision: str = "fp64"):
        """tsdrg.py:500-528; all tensors live on ``device`` (default: current CUDA device).

        ``precision`` for blocks above 64 states (smaller blocks are dense FP64 Jacobi solves):
        'fp64' (default) runs the Kronecker subspace iteration in FP32 and finishes it in FP64,
        matching the reference's FP64 eigh; 'mixed' stops after the FP32 iteration (+ FP64
        Rayleigh-Ritz), several times faster with kept spectra accurate to ~1e-7 relative on
        large clustered blocks."""
        self._mpo = mpo
        self._chi = int(chi)
        self._dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._chain = _Chain(mpo, self._chi, self._dev, precision)

    @property
    def mpo(self) -> MatrixProductOperator:
        return self._mpo

    @property
    def chi(self) -> int:
        return self._chi

    @property
    def tree(self) -> TensorTree:
        return self._chain.tree

    @property
    def n_sites(self) -> int:
        return self._mpo.n_sites

    @property
    def evals(self):
        """Lowest min(chi, m) eigenvalues of the last solved block (numpy), None before run."""
        return self._chain.evals

    def run(self):
        run_chains([self._chain], self._dev)

    @property
    def measurements(self):
        """TreeTensorNetworkMeasurements of the finished tree (tsdrg.py:698-708)."""
        if not self._chain.done:
            raise RuntimeError("tSDRG algorithm hasn't been executed yet.")
        from .tsdrg_measurements import TreeTensorNetworkMeasurements

        return TreeTensorNetworkMeasurements(self._chain.tree, phys_dim=self._mpo.phys_dim, device=self._dev)


TSDRG = TreeTensorNetworkSDRG


class HighEnergyTreeTensorNetworkSDRG(TreeTensorNetworkSDRG):
    """tSDRG keeping the chi highest pairs of every block (tsdrg.py:1031-1067): blocks are
    solved in full by the batched dense Jacobi kernel; the gap is the high-energy one."""

    def __init__(self, mpo: MatrixProductOperator, chi: int, device=None):
        super().__init__(mpo, chi, device=device)
        self._chain = _Chain(mpo, self._chi, self._dev, "fp64", mode="highest")


class ShiftInvertTreeTensorNetworkSDRG(TreeTensorNetworkSDRG):
    """Shift-invert tSDRG (tsdrg.py:1070-1089) for the MPO of H - offset: each block keeps the
    chi pairs of smallest 1/E (the states just below the offset first), reported as E + offset
    in ascending order, with the vectors H x of the generalised problem (unit norm, sign(E) v)."""

    def __init__(self, mpo: MatrixProductOperator, chi: int, offset: float, device=None):
        super().__init__(mpo, chi, device=device)
        self._offset = float(offset)
        self._chain = _Chain(mpo, self._chi, self._dev, "fp64", mode="shift_invert", offset=self._offset)

    @property
    def offset(self) -> float:
        return self._offset


class BatchedTSDRG:
    """Many independent tSDRG chains (e.g. disorder realisations) merged in lockstep:
    every step is one launch of the block-Hamiltonian, eigensolver and projector kernels
    over all chains."""

    def __init__(self, mpos: Sequence[MatrixProductOperator], chi: int, device=None, precision: str = "fp64"):
        self._dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.chi = int(chi)
        self.chains = [_Chain(m, self.chi, self._dev, precision) for m in mpos]

    def run(self):
        run_chains(self.chains, self._dev)
        return self

    @property
    def evals(self) -> list:
        return [c.evals for c in self.chains]

    @property
    def merges(self) -> list:
        return [[(n.left.node_id, n.right.node_id, n.node_id) for n in c.tree if not n.is_leaf] for c in self.chains]
