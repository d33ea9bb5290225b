"""Device-resident MPS and environments (tnpy/matrix_product_state.py).

Every site tensor lives on the GPU as a contiguous FP64 torch tensor of shape
(chi_l, d, chi_r) -- the reference's 'lpr' order (:45) with 1-sized bonds on
the open ends. ``mps[site]`` returns the reference-shaped view: (d, chi) on
site 0, (chi, d) on site n-1. Environments are (ket, mpo, bra) tensors, with
1x1x1 ones on the open ends standing in for the missing L / R of the boundary
sites (:306-307, :425-430).
"""
from __future__ import annotations

from enum import Enum
from pathlib import Path

import numpy as np
import torch

from . import kernels as K
from .operators import MatrixProductOperator


class Direction(Enum):
    """tnpy/matrix_product_state.py:19-25."""

    RIGHTWARD = 1
    LEFTWARD = -1


def bond_dims(n: int, chi: int, d: int) -> list[int]:
    """min(d^i, chi, d^(n-i)): the bond sizes of tnpy's compressed random MPS."""
    return [int(min(d**i, chi, d ** (n - i))) if 0 < i < n else 1 for i in range(n + 1)]


def _device(device) -> torch.device:
    if device is None:
        if not torch.cuda.is_available():
            raise RuntimeError("tnpy_gb300 runs on a CUDA device only")
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device(device)


class MatrixProductState:
    def __init__(self, tensors, device=None):
        """tensors: list of arrays/tensors in 'lpr' order; boundary tensors may be 2-D
        ((d, chi) / (chi, d), the reference's shapes) or 3-D with 1-sized ends."""
        dev = _device(device)
        n = len(tensors)
        if n < 2:
            raise ValueError("an MPS needs at least two sites")
        self._t: list[torch.Tensor] = []
        for s, a in enumerate(tensors):
            t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.asarray(a, dtype=float))
            t = t.to(device=dev, dtype=torch.float64)
            if t.ndim == 2:
                t = t[None] if s == 0 else t[:, :, None]
            if t.ndim != 3:
                raise ValueError(f"site {s}: expected a 2- or 3-index tensor, got {tuple(t.shape)}")
            self._t.append(t.contiguous())
        for s in range(n - 1):
            if self._t[s].shape[2] != self._t[s + 1].shape[0]:
                raise ValueError(f"bond {s}-{s + 1} mismatch")
        self.device = dev

    # ---- structure -------------------------------------------------------------------
    @property
    def n_sites(self) -> int:
        return len(self._t)

    nsites = n_sites

    @property
    def phys_dim(self) -> int:
        return self._t[0].shape[1]

    @property
    def bond_dim(self) -> int:
        return max(t.shape[2] for t in self._t[:-1])

    def bond_dims(self) -> list[int]:
        return [t.shape[2] for t in self._t[:-1]]

    @property
    def tensors(self) -> list[torch.Tensor]:
        """Uniform (chi_l, d, chi_r) device tensors (shared, not copies)."""
        return self._t

    def __getitem__(self, site: int) -> torch.Tensor:
        site = site % self.n_sites
        t = self._t[site]
        if site == 0:
            return t[0]
        if site == self.n_sites - 1:
            return t[:, :, 0]
        return t

    def __iter__(self):
        return (self[s] for s in range(self.n_sites))

    def __len__(self):
        return self.n_sites

    def set_site(self, site: int, data: torch.Tensor):
        t = self._t[site]
        self._t[site] = data.reshape(t.shape).to(device=t.device, dtype=torch.float64).contiguous()

    def to_numpy(self) -> list[np.ndarray]:
        return [t.cpu().numpy() for t in self._t]

    # ---- construction / IO -----------------------------------------------------------
    @classmethod
    def random(cls, n: int, bond_dim: int, phys_dim: int, seed: int | None = 1234, device=None):
        """Seeded N(0,1) tensors with bonds min(d^i, chi, d^(n-i)), right-canonicalised on
        the device and normalised (stands in for the unseeded quimb MPS_rand_state +
        compress of matrix_product_state.py:170-185; the orthogonality centre is site 0,
        where FiniteDMRG.run starts its first, rightward, sweep)."""
        rng = np.random.RandomState(seed)
        dims = bond_dims(n, bond_dim, phys_dim)
        arrays = [rng.standard_normal((dims[i], phys_dim, dims[i + 1])) for i in range(n)]
        mps = cls(arrays, device=device)
        mps.right_canonicalize()
        return mps

    def right_canonicalize(self):
        """Right-canonical form with a normalised centre on site 0. The pushed factor is
        rescaled to unit norm at every step: the norm of a product of ~n random tensors would
        otherwise overflow FP64 on long chains (n = 200 at chi = 512)."""
        for site in range(self.n_sites - 1, 0, -1):
            K.gauge_move(-1, self._t[site], self._t[site - 1])
            self._t[site - 1] /= torch.linalg.vector_norm(self._t[site - 1])

    def left_canonicalize(self):
        for site in range(self.n_sites - 1):
            K.gauge_move(1, self._t[site], self._t[site + 1])
            self._t[site + 1] /= torch.linalg.vector_norm(self._t[site + 1])

    def save(self, filename: str):
        """Reference-shaped tensors in site order to ``.npz`` (matrix_product_state.py:118-142;
        ``.hdf5`` needs h5py, which the library does not use)."""
        path = Path(filename)
        if path.suffix != ".npz":
            raise ValueError(f"File extension {path.suffix} is not supported.")
        np.savez(str(path), **{f"I{s}": self[s].cpu().numpy() for s in range(self.n_sites)})

    @classmethod
    def load(cls, filename: str, device=None):
        path = Path(filename)
        if path.suffix != ".npz":
            raise ValueError(f"File extension {path.suffix} is not supported.")
        f = np.load(str(path))
        keys = sorted(f.files, key=lambda k: int(k[1:]))
        return cls([f[k] for k in keys], device=device)

    # ---- gauge move ------------------------------------------------------------------
    def split_tensor(self, site: int, direction: Direction, precision="fp64"):
        """Gauge move onto the neighbour (QR form of matrix_product_state.py:187-225)."""
        if direction == Direction.RIGHTWARD:
            K.gauge_move(1, self._t[site], self._t[site + 1], precision=precision)
        elif direction == Direction.LEFTWARD:
            K.gauge_move(-1, self._t[site], self._t[site - 1], precision=precision)
        else:
            raise KeyError("MatrixProductState only supplies left or right direction.")

    def enlarge_bond_dim(self, new_bond_dim: int, method: str = "random", seed: int | None = 0):
        """Grow every bond to min(d^i, new_bond_dim, d^(n-i)) without changing the state
        (the reference's stub, matrix_product_state.py:227-228, returns NotImplemented).

        The MPS must be right-canonical with its centre on site 0 (the state after a leftward
        sweep or ``random``). Bonds are grown from the right: site i+1 gains new rows that are
        random directions orthogonalised (Householder QR on the device) against its existing
        rows, and site i gains matching zero columns, so the state and the right-canonical form
        are unchanged while one-site sweeps can populate the new directions. Used for the
        bond-dimension ramp of one-site DMRG."""
        if method != "random":
            raise ValueError(f"unknown enlargement method {method!r}")
        n, d = self.n_sites, self.phys_dim
        target = bond_dims(n, new_bond_dim, d)
        gen = torch.Generator(device="cpu")
        gen.manual_seed(0 if seed is None else int(seed))
        for i in range(n - 2, -1, -1):  # bond between sites i and i+1
            a, b = self._t[i], self._t[i + 1]
            old, new = b.shape[0], target[i + 1]
            if new <= old:
                continue
            rows = b.reshape(old, -1)  # orthonormal rows (right-canonical)
            extra = torch.randn(new - old, rows.shape[1], generator=gen, dtype=torch.float64).to(self.device)
            m = torch.cat([rows, extra], 0).T.contiguous()  # (d chi_r) x new
            q, _ = K.qr(m)
            grown = torch.cat([rows, q[:, old:].T], 0)
            self._t[i + 1] = grown.reshape(new, d, b.shape[2]).contiguous()
            pad = torch.zeros(a.shape[0], d, new - old, dtype=torch.float64, device=self.device)
            self._t[i] = torch.cat([a, pad], 2).contiguous()
        return self

    def conj(self) -> "MatrixProductState":
        return MatrixProductState([t.clone() for t in self._t], device=self.device)


class OneSiteOperator:
    """Matrix-free H_eff of one site: the drop-in for the scipy LinearOperator returned by
    Environment.one_site_matvec (matrix_product_state.py:411-440)."""

    def __init__(self, left, w, right, shape, precision="fp64"):
        self.left, self.w, self.right = left, w, right
        self.site_shape = shape
        n = int(np.prod(shape))
        self.shape = (n, n)
        self.dtype = np.float64
        self.precision = precision

    def matvec(self, x):
        as_numpy = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, dtype=float)) if as_numpy else x
        xt = xt.to(device=self.left.device, dtype=torch.float64).reshape(self.site_shape).contiguous()
        y = K.matvec1(self.left, self.w, self.right, xt, precision=self.precision)
        y = y.reshape(-1, 1)
        return y.cpu().numpy() if as_numpy else y

    __matmul__ = matvec


class Environment:
    def __init__(self, mpo: MatrixProductOperator, mps: MatrixProductState, precision="fp64",
                 env_dtype: torch.dtype = torch.float64):
        """Left / right environments of ``mps`` under ``mpo`` (matrix_product_state.py:231-250).

        ``precision`` selects the contraction kernels of the environment updates and gauge
        moves: 'fp64' native FP64; 'mixed' (and 'df64') FP64-class arithmetic. ``env_dtype``
        is the storage type of the environments: float64, or float32 (half the resident
        bytes; each environment is computed in the contraction's arithmetic and rounded to
        FP32 when stored, and widened back to FP64 when a site's operator is read)."""
        if mpo.n_sites != mps.n_sites:
            raise ValueError("MPO and MPS sizes differ")
        if env_dtype not in (torch.float64, torch.float32):
            raise ValueError(f"environments are stored as float64 or float32, not {env_dtype}")
        self._mpo = mpo
        self._mps = mps
        self._n_sites = mps.n_sites
        self._w = mpo.device_tensors(mps.device)
        self.precision = precision
        self.env_dtype = env_dtype
        self.rebuild()

    def close(self):
        del self._left, self._right

    def rebuild(self):
        """Recompute every environment (after the bond dimensions changed)."""
        one = torch.ones((1, 1, 1), dtype=self.env_dtype, device=self._mps.device)
        self._left = {0: one}
        self._right = {self._n_sites - 1: one.clone()}
        for site in range(1, self._n_sites):
            self.update_left(site)
        for site in range(self._n_sites - 2, -1, -1):
            self.update_right(site)

    def _f64(self, t: torch.Tensor) -> torch.Tensor:
        return t if t.dtype == torch.float64 else t.to(torch.float64)

    def _store(self, store: dict, site: int, e: torch.Tensor):
        if self.env_dtype == torch.float64:
            store[site] = e
        else:
            old = store.get(site)
            if old is not None and old.shape == e.shape:
                old.copy_(e)
            else:
                store[site] = e.to(self.env_dtype)

    @property
    def mpo(self) -> MatrixProductOperator:
        return self._mpo

    @property
    def mps(self) -> MatrixProductState:
        return self._mps

    @property
    def n_sites(self) -> int:
        return self._n_sites

    @property
    def left(self) -> dict[int, torch.Tensor]:
        return self._left

    @property
    def right(self) -> dict[int, torch.Tensor]:
        return self._right

    def update_left(self, site: int):
        """L_site from L_{site-1}, A_{site-1}, W_{site-1} (:296-315)."""
        a = self._mps.tensors[site - 1]
        out = self._left.get(site) if self.env_dtype == torch.float64 else None
        shape = (a.shape[2], self._w[site - 1].shape[1], a.shape[2])
        if out is None or tuple(out.shape) != shape:
            out = None
        e = K.env_update(1, self._f64(self._left[site - 1]), a, self._w[site - 1], out=out,
                         precision=self.precision)
        self._store(self._left, site, e)

    def update_right(self, site: int):
        """R_site from R_{site+1}, A_{site+1}, W_{site+1} (:317-336)."""
        a = self._mps.tensors[site + 1]
        out = self._right.get(site) if self.env_dtype == torch.float64 else None
        shape = (a.shape[0], self._w[site + 1].shape[0], a.shape[0])
        if out is None or tuple(out.shape) != shape:
            out = None
        e = K.env_update(-1, self._f64(self._right[site + 1]), a, self._w[site + 1], out=out,
                         precision=self.precision)
        self._store(self._right, site, e)

    def update(self, site: int, direction: Direction):
        """:338-353."""
        if direction == Direction.RIGHTWARD:
            self.update_left(site + 1)
        elif direction == Direction.LEFTWARD:
            self.update_right(site - 1)

    def update_mps(self, site: int, data):
        """:355-357 (the bra is the same tensor here, so one write updates both)."""
        if not isinstance(data, torch.Tensor):
            data = torch.as_tensor(np.asarray(data, dtype=float))
        self._mps.set_site(site, data)

    def split_tensor(self, site: int, direction: Direction):
        """:359-365."""
        self._mps.split_tensor(site, direction, precision=self.precision)

    def one_site_full_matrix(self, site: int) -> torch.Tensor:
        """Dense H_eff, rows = ket (:372-409)."""
        return K.full_matrix1(self._f64(self._left[site]), self._w[site], self._f64(self._right[site]))

    def one_site_matvec(self, site: int, precision=None) -> OneSiteOperator:
        return OneSiteOperator(self._f64(self._left[site]), self._w[site], self._f64(self._right[site]),
                               tuple(self._mps.tensors[site].shape),
                               precision=precision or "fp64")

    def site_operator(self, site: int):
        """(L, W, R) of ``site`` as FP64 device tensors."""
        return self._f64(self._left[site]), self._w[site], self._f64(self._right[site])

    def variance(self) -> float:
        """<H^2> - <H>^2 on the current (unnormalised) MPS (:367-370)."""
        return expectation_value(self._mps, self._mpo.square()) - expectation_value(self._mps, self._mpo) ** 2


def expectation_value(mps: MatrixProductState, mpo: MatrixProductOperator | None = None) -> float:
    """<psi|O|psi> (or <psi|psi>) by a left-to-right environment sweep on the device."""
    if mpo is None:
        d = mps.phys_dim
        ident = np.zeros((1, 1, d, d))
        ident[0, 0] = np.eye(d)
        mpo_t = [torch.from_numpy(ident).to(mps.device)] * mps.n_sites
    else:
        mpo_t = mpo.device_tensors(mps.device)
    env = torch.ones((1, 1, 1), dtype=torch.float64, device=mps.device)
    for a, w in zip(mps.tensors, mpo_t):
        env = K.env_update(1, env, a, w)
    return float(env.reshape(-1)[0].item())


class MatrixProductStateMeasurements:
    """tnpy/matrix_product_state.py:443-453."""

    def __init__(self, mps: MatrixProductState):
        self._mps = mps

    def expectation_value(self, mpo: MatrixProductOperator | None = None) -> float:
        return expectation_value(self._mps, mpo)

    def local_sz(self) -> np.ndarray:
        """<Sz_i> / <psi|psi> for every site: left / right norm environments (identity MPO)
        once, then one D=1 matvec with W = Sz per site, all on the device."""
        mps = self._mps
        n, d, dev = mps.n_sites, mps.phys_dim, mps.device
        eye = torch.eye(d, dtype=torch.float64, device=dev).reshape(1, 1, d, d).contiguous()
        sz = torch.diag(torch.tensor([0.5 * (d - 1) - k for k in range(d)], dtype=torch.float64,
                                     device=dev)).reshape(1, 1, d, d).contiguous()
        one = torch.ones((1, 1, 1), dtype=torch.float64, device=dev)
        lefts = [one]
        for a in mps.tensors[:-1]:
            lefts.append(K.env_update(1, lefts[-1], a, eye))
        rights = [one]
        for a in mps.tensors[:0:-1]:
            rights.append(K.env_update(-1, rights[-1], a, eye))
        rights = rights[::-1]
        out = torch.empty(n, dtype=torch.float64, device=dev)
        a0 = mps.tensors[0]
        nrm = torch.dot(a0.reshape(-1), K.matvec1(lefts[0], eye, rights[0], a0).reshape(-1))
        for i, a in enumerate(mps.tensors):
            out[i] = torch.dot(a.reshape(-1), K.matvec1(lefts[i], sz, rights[i], a).reshape(-1))
        return (out / nrm).cpu().numpy()

    def schmidt_values(self, bond: int) -> torch.Tensor:
        """Schmidt values on ``bond`` (between sites bond and bond+1) of the normalised state,
        largest first, as a device tensor. A copy of the MPS is gauged with the orthogonality
        centre on site ``bond`` (Householder QR moves from both ends, FP64), and the singular
        values of the centre tensor reshaped to (chi_l d, chi_r) are computed directly by
        Householder QR and a one-sided Jacobi SVD of R: the singular values of the SVD gauge
        move (matrix_product_state.py:200-223) at that bond. No Gram matrix is formed, so the
        small values keep an absolute error of ~eps * s_max."""
        mps = self._mps
        n = mps.n_sites
        if not 0 <= bond < n - 1:
            raise ValueError(f"bond {bond} is not between two sites of a {n}-site chain")
        t = [a.clone() for a in mps.tensors]
        for site in range(bond):
            K.gauge_move(1, t[site], t[site + 1])
        for site in range(n - 1, bond, -1):
            K.gauge_move(-1, t[site], t[site - 1])
        c = t[bond]
        cl, d, cr = c.shape
        m = c.reshape(cl * d, cr)
        if m.shape[0] < m.shape[1]:
            m = m.T.contiguous()
        _, r = K.qr(m)
        _, sv, _ = K.svd(r, want_u=False, want_vt=False)
        return sv / torch.linalg.vector_norm(sv)

    def entanglement_spectrum(self, bond: int) -> np.ndarray:
        """Schmidt values on ``bond`` (``schmidt_values``) as a host array: the entanglement
        spectrum's lambda_k, with sum lambda_k^2 = 1."""
        return self.schmidt_values(bond).cpu().numpy()
