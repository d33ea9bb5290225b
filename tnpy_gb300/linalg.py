"""tnpy.linalg call shapes over device tensors (tnpy/linalg.py:9-87).

``svd`` / ``qr`` / ``eigh`` / ``eigshmv`` keep the reference's arguments and
return shapes, run on the GPU through libtnx and return torch CUDA tensors
(numpy inputs are copied to the current device first).
"""
from __future__ import annotations

import numpy as np
import torch

from . import kernels as K


def _dev(matrix) -> torch.Tensor:
    if isinstance(matrix, torch.Tensor):
        t = matrix
    else:
        t = torch.as_tensor(np.asarray(matrix, dtype=float))
    if not t.is_cuda:
        t = t.to(torch.device("cuda", torch.cuda.current_device()))
    return t.to(torch.float64).contiguous()


def qr(matrix, cutoff: int):
    """Reduced QR sliced to ``cutoff`` (linalg.py:26-39). Householder, FP64, on the device;
    for m < n the transposed problem is factored (Q R = M with Q square)."""
    m = _dev(matrix)
    rows, cols = m.shape
    if rows >= cols:
        q, r = K.qr(m)
    else:
        # M = [M1 M2] with M1 square: Q R1 = M1, R = Q^T M
        q, _ = K.qr(m[:, :rows].contiguous())
        r = K.gemm(q, m, trans_a=True)
    return q[:, :cutoff].contiguous(), r[:cutoff, :].contiguous()


def eigh(matrix, k: int = 1, backend: str = "numpy", **kwargs):
    """Lowest k eigenpairs of a symmetric matrix (linalg.py:42-61); k=1 returns
    (float, vector), otherwise (evals[:k], evecs[:, :k]). ``backend`` is accepted for
    call-shape compatibility; generalised problems (``b=``) are not part of this path."""
    if "b" in kwargs and kwargs["b"] is not None:
        raise NotImplementedError("generalised eigenproblems (b=) are outside the DMRG/tSDRG path")
    if backend not in ("numpy", "scipy"):
        raise KeyError(backend)
    a = _dev(matrix)
    n = a.shape[0]
    keep = n if k is None else min(int(k), n)
    evals, evecs = K.eigh_batched([a], keep=keep)
    evals, evecs = evals[0], evecs[0, :n, :]
    if k == 1:
        return float(evals[0].item()), evecs[:, 0]
    return evals, evecs


def svd(matrix, cutoff: int):
    """Reduced SVD sliced to ``cutoff`` (linalg.py:9-23): Householder QR (M = Q R) and a
    one-sided Jacobi SVD of R (R = U_r S V^T) on the device, U = Q U_r, all in FP64. The singular
    values come from R itself, so a small singular value keeps an absolute error of
    ~eps * s_max (a Gram matrix R R^T would leave ~sqrt(eps) * s_max), and U, V^T are orthonormal
    to working accuracy. Columns of U whose singular value is exactly zero are completed to an
    orthonormal set (np.linalg.svd does the same)."""
    m = _dev(matrix)
    rows, cols = m.shape
    if rows < cols:
        u, s, vt = svd(m.T.contiguous(), cutoff)
        return vt.T.contiguous(), s, u.T.contiguous()
    q, r = K.qr(m)  # m = Q R, R cols x cols
    ur, s, vt = K.svd(r)
    u = K.gemm(q, ur)
    zero = (s == 0).nonzero().flatten()
    if zero.numel():
        u = _complete_columns(u, zero)
    return u[:, :cutoff].contiguous(), s[:cutoff].contiguous(), vt[:cutoff, :].contiguous()


def _complete_columns(u: torch.Tensor, cols: torch.Tensor) -> torch.Tensor:
    """Replace the given (zero) columns of u, whose other columns are orthonormal, by unit
    vectors orthogonal to everything else: seeded random fill, Householder QR, signs of the
    kept columns restored from diag(R)."""
    g = torch.Generator(device="cpu").manual_seed(0)
    u = u.clone()
    u[:, cols] = torch.randn((u.shape[0], cols.numel()), generator=g, dtype=torch.float64).to(u.device)
    q, r = K.qr(u.contiguous())
    sign = torch.where(torch.diagonal(r) < 0, -1.0, 1.0).to(torch.float64)
    return (q * sign[None, :]).contiguous()


def eigshmv(linear_operator, v0, k: int = 1, which: str = "SA", tol: float = 0, **kwargs):
    """Lowest eigenpair of a one-site effective Hamiltonian (linalg.py:64-87).

    ``linear_operator`` is the object returned by ``Environment.one_site_matvec``; the
    device Davidson replaces primme. Returns (eigenvalue, eigenvector of shape (N, 1)).
    Extra keyword arguments: ``max_iter``, ``max_basis``, ``precision``; other primme
    options are accepted and ignored."""
    from .matrix_product_state import OneSiteOperator

    if k != 1 or which != "SA":
        raise NotImplementedError("only the lowest eigenpair (k=1, which='SA') is on this path")
    if not isinstance(linear_operator, OneSiteOperator):
        raise TypeError("eigshmv takes the operator returned by Environment.one_site_matvec")
    x = _dev(v0).reshape(linear_operator.site_shape).clone()
    tol = float(tol) if tol else 1e-12
    e, _, _, _ = K.davidson1(linear_operator.left, linear_operator.w, linear_operator.right, x, tol=tol,
                             max_iter=int(kwargs.get("max_iter", 400)),
                             max_basis=int(kwargs.get("max_basis", 24)),
                             precision=kwargs.get("precision", linear_operator.precision))
    return e, x.reshape(-1, 1)
