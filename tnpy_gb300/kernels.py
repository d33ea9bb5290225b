"""Typed wrappers of the tnx C ABI over torch CUDA tensors.

Each wrapper checks shapes on the host, takes scratch from the per-device
workspace and calls exactly one C entry point on the current torch stream.
Layouts follow include/tnx.h: MPS A[chi_l, d, chi_r], MPO W[dl, dr, d, d],
environments E[chi, D, chi] (ket, mpo, bra).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import check, lib, ptr, stream_ptr, Workspace


def _f64(t: torch.Tensor, name: str) -> torch.Tensor:
    if t.dtype != torch.float64:
        raise ValueError(f"{name} must be float64 (got {t.dtype})")
    if not t.is_cuda:
        raise ValueError(f"{name} must live on a CUDA device")
    return t.contiguous()


def _site_dims(L, W, R):
    chi_l, dl, chi_l2 = L.shape
    dl2, dr, d, d2 = W.shape
    chi_r, dr2, chi_r2 = R.shape
    if chi_l != chi_l2 or chi_r != chi_r2 or dl != dl2 or dr != dr2 or d != d2:
        raise ValueError(f"inconsistent L {tuple(L.shape)}, W {tuple(W.shape)}, R {tuple(R.shape)}")
    return chi_l, d, chi_r, dl, dr


def precision_code(precision) -> int:
    if isinstance(precision, int):
        return precision
    try:
        return _lib.PRECISIONS[precision]
    except KeyError:
        raise ValueError(f"unknown precision {precision!r}; use 'fp64' or 'mixed'") from None


def matvec1(L, W, R, x, y=None, precision="fp64"):
    """y = H_eff x for one site (Environment.one_site_matvec, matrix_product_state.py:411-440)."""
    L, W, R, x = (_f64(t, n) for t, n in ((L, "L"), (W, "W"), (R, "R"), (x, "x")))
    chi_l, d, chi_r, dl, dr = _site_dims(L, W, R)
    if x.numel() != chi_l * d * chi_r:
        raise ValueError(f"x has {x.numel()} elements, expected {chi_l * d * chi_r}")
    if y is None:
        y = torch.empty((chi_l, d, chi_r), dtype=torch.float64, device=x.device)
    p = precision_code(precision)
    nbytes = lib.tnx_matvec1_workspace_bytes(chi_l, d, chi_r, dl, dr, p)
    wp, wn = Workspace.get(nbytes, x.device)
    check("tnx_matvec1", lib.tnx_matvec1(ptr(L), ptr(W), ptr(R), ptr(x), ptr(y), chi_l, d, chi_r, dl, dr,
                                         p, wp, wn, stream_ptr()))
    return y


def full_matrix1(L, W, R):
    """Dense H_eff[(a,s,c),(a',s',c')] (Environment.one_site_full_matrix, :372-409)."""
    L, W, R = _f64(L, "L"), _f64(W, "W"), _f64(R, "R")
    chi_l, d, chi_r, dl, dr = _site_dims(L, W, R)
    n = chi_l * d * chi_r
    H = torch.empty((n, n), dtype=torch.float64, device=L.device)
    check("tnx_full_matrix1", lib.tnx_full_matrix1(ptr(L), ptr(W), ptr(R), ptr(H), chi_l, d, chi_r, dl, dr,
                                                   stream_ptr()))
    return H


def diag1(L, W, R):
    L, W, R = _f64(L, "L"), _f64(W, "W"), _f64(R, "R")
    chi_l, d, chi_r, dl, dr = _site_dims(L, W, R)
    out = torch.empty((chi_l, d, chi_r), dtype=torch.float64, device=L.device)
    check("tnx_diag1", lib.tnx_diag1(ptr(L), ptr(W), ptr(R), ptr(out), chi_l, d, chi_r, dl, dr, stream_ptr()))
    return out


def env_update(direction: int, E, A, W, out=None, precision="fp64"):
    """L_{i+1} from L_i (direction +1) or R_{i-1} from R_i (-1) (matrix_product_state.py:296-336)."""
    E, A, W = _f64(E, "E"), _f64(A, "A"), _f64(W, "W")
    chi_l, d, chi_r = A.shape
    dl, dr = W.shape[0], W.shape[1]
    if direction == 1:
        if tuple(E.shape) != (chi_l, dl, chi_l):
            raise ValueError(f"left environment {tuple(E.shape)} does not match A {tuple(A.shape)} / W")
        shape = (chi_r, dr, chi_r)
    elif direction == -1:
        if tuple(E.shape) != (chi_r, dr, chi_r):
            raise ValueError(f"right environment {tuple(E.shape)} does not match A {tuple(A.shape)} / W")
        shape = (chi_l, dl, chi_l)
    else:
        raise KeyError("direction must be +1 (rightward) or -1 (leftward)")
    if out is None:
        out = torch.empty(shape, dtype=torch.float64, device=A.device)
    p = precision_code(precision)
    nbytes = lib.tnx_env_update_workspace_bytes(direction, chi_l, d, chi_r, dl, dr, p)
    wp, wn = Workspace.get(nbytes, A.device)
    check("tnx_env_update", lib.tnx_env_update(direction, ptr(E), ptr(A), ptr(W), ptr(out), chi_l, d, chi_r,
                                               dl, dr, p, wp, wn, stream_ptr()))
    return out


def davidson1(L, W, R, x, tol=1e-8, max_iter=200, max_basis=24, precision="fp64", raise_on_fail=False,
              start_anchored=False):
    """Lowest eigenpair of H_eff starting from x (overwritten with the unit eigenvector).

    ``start_anchored`` (mixed precision): x is expected to be the answer already; the solve
    starts with the FP64-class anchor product instead of a split-BF16 phase.
    Returns (eigenvalue, residual norm, matvec count, converged)."""
    L, W, R = _f64(L, "L"), _f64(W, "W"), _f64(R, "R")
    if x.dtype != torch.float64 or not x.is_cuda or not x.is_contiguous():
        raise ValueError("x must be a contiguous float64 CUDA tensor (it is overwritten)")
    chi_l, d, chi_r, dl, dr = _site_dims(L, W, R)
    p = precision_code(precision)
    nbytes = lib.tnx_davidson1_workspace_bytes(chi_l, d, chi_r, dl, dr, max_basis, p)
    wp, wn = Workspace.get(nbytes, x.device)
    ev = ctypes.c_double(0.0)
    rn = ctypes.c_double(0.0)
    it = ctypes.c_int(0)
    st = lib.tnx_davidson1_ex(ptr(L), ptr(W), ptr(R), ptr(x), chi_l, d, chi_r, dl, dr, float(tol), int(max_iter),
                              int(max_basis), p, 1 if start_anchored else 0, ctypes.byref(ev), ctypes.byref(rn),
                              ctypes.byref(it), wp, wn, stream_ptr())
    converged = st == _lib.TNX_OK
    if st != _lib.TNX_OK and (st != _lib.TNX_ERR_NOT_CONVERGED or raise_on_fail):
        check("tnx_davidson1", st)
    return ev.value, rn.value, it.value, converged


def gdavidson1(L, W, R, L2, W2, R2, x, tol=1e-8, max_iter=400, max_basis=24, precision="fp64"):
    """Lowest eigenpair of A x = lambda B x with A = H_eff(L, W, R), B = H_eff(L2, W2, R2)
    (B positive definite) from x (overwritten with the B-unit eigenvector).
    Returns (eigenvalue, residual norm, expansions, converged)."""
    L, W, R, L2, W2, R2 = (_f64(t, n) for t, n in ((L, "L"), (W, "W"), (R, "R"), (L2, "L2"), (W2, "W2"), (R2, "R2")))
    if x.dtype != torch.float64 or not x.is_cuda or not x.is_contiguous():
        raise ValueError("x must be a contiguous float64 CUDA tensor (it is overwritten)")
    chi_l, d, chi_r, dl, dr = _site_dims(L, W, R)
    chi_l2, d2, chi_r2, dl2, dr2 = _site_dims(L2, W2, R2)
    if (chi_l2, d2, chi_r2) != (chi_l, d, chi_r):
        raise ValueError("the two operators act on different site shapes")
    p = precision_code(precision)
    wp, wn = Workspace.get(lib.tnx_gdavidson1_workspace_bytes(chi_l, d, chi_r, dl, dr, dl2, dr2, max_basis), x.device)
    ev, rn, it = ctypes.c_double(0.0), ctypes.c_double(0.0), ctypes.c_int(0)
    st = lib.tnx_gdavidson1(ptr(L), ptr(W), ptr(R), ptr(L2), ptr(W2), ptr(R2), ptr(x), chi_l, d, chi_r, dl, dr, dl2,
                            dr2, float(tol), int(max_iter), int(max_basis), p, ctypes.byref(ev), ctypes.byref(rn),
                            ctypes.byref(it), wp, wn, stream_ptr())
    if st not in (_lib.TNX_OK, _lib.TNX_ERR_NOT_CONVERGED):
        check("tnx_gdavidson1", st)
    return ev.value, rn.value, it.value, st == _lib.TNX_OK


def mpo_apply_site(A: torch.Tensor, W: torch.Tensor) -> torch.Tensor:
    """out[(a w), k, (c v)] = sum_b W[w, v, k, b] A[a, b, c]: one site of O|psi>."""
    A, W = _f64(A, "A"), _f64(W, "W")
    chi_l, d, chi_r = A.shape
    dl, dr = W.shape[0], W.shape[1]
    out = torch.empty((chi_l * dl, d, chi_r * dr), dtype=torch.float64, device=A.device)
    check("tnx_mpo_apply_site", lib.tnx_mpo_apply_site(ptr(A), ptr(W), ptr(out), chi_l, d, chi_r, dl, dr,
                                                       stream_ptr()))
    return out


def davidson1_stats() -> dict:
    """Counters of this thread's last davidson1 call: first-phase matvecs, anchored-phase
    matvecs (mixed form), FP64-class anchor products and thick restarts."""
    out = (ctypes.c_int * 4)()
    check("tnx_davidson1_stats", lib.tnx_davidson1_stats(out))
    return {"phase1": out[0], "anchored": out[1], "anchors": out[2], "restarts": out[3]}


def eigh_batched(mats: list[torch.Tensor], keep: int, precision: str = "fp64"):
    """Lowest `keep` eigenpairs of each symmetric matrix (one CTA per matrix).

    Returns (evals [batch, keep], evecs [batch, max_size, keep]); for a matrix smaller than
    `keep` only its own eigenpairs are written (the rest is NaN / zero). precision 'df64':
    double-FP32 Jacobi in shared memory for matrices up to 64 rows (FP64 above)."""
    if not mats:
        raise ValueError("no matrices")
    dev = mats[0].device
    sizes = [int(m.shape[0]) for m in mats]
    for m in mats:
        if m.ndim != 2 or m.shape[0] != m.shape[1]:
            raise ValueError(f"matrix of shape {tuple(m.shape)} is not square")
    if keep > max(sizes):
        raise ValueError(f"keep={keep} exceeds the largest matrix ({max(sizes)})")
    offs, o = [], 0
    for s in sizes:
        offs.append(o)
        o += s * s
    packed = torch.cat([_f64(m, "matrix").reshape(-1) for m in mats])
    max_size = max(sizes)
    batch = len(mats)
    offsets = torch.tensor(offs, dtype=torch.int64, device=dev)
    sizes_t = torch.tensor(sizes, dtype=torch.int32, device=dev)
    evals = torch.full((batch, keep), float("nan"), dtype=torch.float64, device=dev)
    evecs = torch.zeros((batch, max_size, keep), dtype=torch.float64, device=dev)
    if precision == "df64" and max_size <= 64:
        check("tnx_eigh_batched_df64", lib.tnx_eigh_batched_df64(ptr(packed), ptr(offsets), ptr(sizes_t), batch,
                                                                 max_size, keep, ptr(evals), ptr(evecs),
                                                                 stream_ptr()))
        return evals, evecs
    nbytes = lib.tnx_eigh_batched_workspace_bytes(batch, max_size, keep)
    wp, wn = Workspace.get(nbytes, dev)
    check("tnx_eigh_batched", lib.tnx_eigh_batched(ptr(packed), ptr(offsets), ptr(sizes_t), batch, max_size,
                                                   keep, ptr(evals), ptr(evecs), wp, wn, stream_ptr()))
    return evals, evecs


def qr(M: torch.Tensor):
    """Reduced Householder QR of an m x n (m >= n) matrix."""
    M = _f64(M, "matrix")
    m, n = M.shape
    Q = torch.empty((m, n), dtype=torch.float64, device=M.device)
    Rm = torch.empty((n, n), dtype=torch.float64, device=M.device)
    wp, wn = Workspace.get(lib.tnx_qr_workspace_bytes(m, n), M.device)
    check("tnx_qr", lib.tnx_qr(ptr(M), m, n, ptr(Q), ptr(Rm), wp, wn, stream_ptr()))
    return Q, Rm


def svd(M: torch.Tensor, want_u: bool = True, want_vt: bool = True):
    """Thin SVD of an m x n (m >= n) matrix by one-sided Jacobi (tnx_svd): (U, S, VT), S
    descending; U / VT are None when not requested."""
    M = _f64(M, "matrix")
    m, n = M.shape
    if m < n:
        raise ValueError(f"svd needs m >= n (got {m} x {n})")
    S = torch.empty(n, dtype=torch.float64, device=M.device)
    U = torch.empty((m, n), dtype=torch.float64, device=M.device) if want_u else None
    VT = torch.empty((n, n), dtype=torch.float64, device=M.device) if want_vt else None
    wp, wn = Workspace.get(lib.tnx_svd_workspace_bytes(m, n, int(want_vt)), M.device)
    sweeps = ctypes.c_int(0)
    check("tnx_svd", lib.tnx_svd(ptr(M), m, n, ptr(S), ptr(U), ptr(VT), ctypes.byref(sweeps), wp, wn,
                                 stream_ptr()))
    return U, S, VT


def gauge_move(direction: int, a_site: torch.Tensor, a_nb: torch.Tensor, precision="fp64"):
    """In-place one-site gauge move (QR form of split_tensor, matrix_product_state.py:187-225)."""
    if not (a_site.is_contiguous() and a_nb.is_contiguous()):
        raise ValueError("MPS tensors must be contiguous")
    chi_l, d, chi_r = a_site.shape
    if direction == 1:
        if a_nb.shape[0] != chi_r:
            raise ValueError("right neighbour does not share the bond")
        other = a_nb.shape[2]
    elif direction == -1:
        if a_nb.shape[2] != chi_l:
            raise ValueError("left neighbour does not share the bond")
        other = a_nb.shape[0]
    else:
        raise KeyError("MatrixProductState only supplies left or right direction.")
    nbytes = lib.tnx_gauge_move_workspace_bytes(direction, chi_l, d, chi_r, other)
    wp, wn = Workspace.get(nbytes, a_site.device)
    check("tnx_gauge_move", lib.tnx_gauge_move(direction, ptr(a_site), ptr(a_nb), chi_l, d, chi_r, other,
                                               precision_code(precision), wp, wn, stream_ptr()))


def gemm(a: torch.Tensor, b: torch.Tensor, trans_a=False, trans_b=False, out=None, alpha=1.0, beta=0.0):
    a, b = _f64(a, "a"), _f64(b, "b")
    m = a.shape[1] if trans_a else a.shape[0]
    k = a.shape[0] if trans_a else a.shape[1]
    n = b.shape[0] if trans_b else b.shape[1]
    kb = b.shape[1] if trans_b else b.shape[0]
    if k != kb:
        raise ValueError("inner dimensions differ")
    if out is None:
        out = torch.zeros((m, n), dtype=torch.float64, device=a.device)
    check("tnx_gemm_f64", lib.tnx_gemm_f64(int(trans_a), int(trans_b), m, n, k, float(alpha), ptr(a),
                                           a.shape[1], 0, ptr(b), b.shape[1], 0, float(beta), ptr(out), n, 0, 1,
                                           stream_ptr()))
    return out


def gemm_bf16x3(a: torch.Tensor, b: torch.Tensor):
    """C = A B^T (A: m x k, B: n x k, FP64 in and out) on the tensor cores, split-BF16."""
    a, b = _f64(a, "a"), _f64(b, "b")
    m, k = a.shape
    n, kb = b.shape
    if k != kb:
        raise ValueError("inner dimensions differ")
    out = torch.empty((m, n), dtype=torch.float64, device=a.device)
    wp, wn = Workspace.get(lib.tnx_gemm_bf16x3_workspace_bytes(m, n, k), a.device)
    check("tnx_gemm_bf16x3", lib.tnx_gemm_bf16x3(m, n, k, ptr(a), ptr(b), ptr(out), wp, wn, stream_ptr()))
    return out


def gemm_df64(a: torch.Tensor, b: torch.Tensor, trans_a=False, trans_b=False):
    """C = op(A) op(B) in double-FP32 arithmetic (FP64 in / out)."""
    a, b = _f64(a, "a"), _f64(b, "b")
    m = a.shape[1] if trans_a else a.shape[0]
    k = a.shape[0] if trans_a else a.shape[1]
    n = b.shape[0] if trans_b else b.shape[1]
    out = torch.empty((m, n), dtype=torch.float64, device=a.device)
    check("tnx_gemm_df64", lib.tnx_gemm_df64(int(trans_a), int(trans_b), m, n, k, 1.0, ptr(a), a.shape[1], ptr(b),
                                             b.shape[1], 0.0, ptr(out), n, stream_ptr()))
    return out


def gemm_oz(a: torch.Tensor, b: torch.Tensor, trans_a=False, trans_b=False):
    """C = op(A) op(B), FP64 in / out, on the tensor cores by exact integer slicing (Ozaki)."""
    a, b = _f64(a, "a"), _f64(b, "b")
    m = a.shape[1] if trans_a else a.shape[0]
    k = a.shape[0] if trans_a else a.shape[1]
    n = b.shape[0] if trans_b else b.shape[1]
    out = torch.empty((m, n), dtype=torch.float64, device=a.device)
    wp, wn = Workspace.get(lib.tnx_gemm_oz_workspace_bytes(m, n, k), a.device)
    check("tnx_gemm_oz", lib.tnx_gemm_oz(int(trans_a), int(trans_b), m, n, k, 1.0, ptr(a), a.shape[1], ptr(b),
                                         b.shape[1], 0.0, ptr(out), n, wp, wn, stream_ptr()))
    return out


def gemm_oz_batched(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor | None = None, *, alpha=1.0, beta=0.0,
                    nsplit: int = 1, mask: torch.Tensor | None = None):
    """C[i] = alpha A[i] B[i] + beta C[i] for stacked [batch, m, k] / [batch, k, n] FP64 tensors in one
    tensor-core launch (Ozaki), K split into `nsplit` ranges; entries with mask[i] == 0 are left
    untouched."""
    a, b = _f64(a, "a"), _f64(b, "b")
    if a.ndim != 3 or b.ndim != 3 or a.shape[0] != b.shape[0] or a.shape[2] != b.shape[1]:
        raise ValueError(f"shapes {tuple(a.shape)} and {tuple(b.shape)} do not form a batched product")
    bt, m, k = a.shape
    n = b.shape[2]
    if c is None:
        c = torch.zeros((bt, m, n), dtype=torch.float64, device=a.device)
    if mask is not None:
        mask = mask.to(device=a.device, dtype=torch.int32).contiguous()
    wp, wn = Workspace.get(lib.tnx_gemm_oz_batched_workspace_bytes(m, n, k, bt, nsplit), a.device)
    check("tnx_gemm_oz_batched",
          lib.tnx_gemm_oz_batched(0, 0, m, n, k, float(alpha), ptr(a), k, m * k, ptr(b), n, k * n, float(beta),
                                  ptr(c), n, m * n, bt, nsplit, ptr(mask) if mask is not None else None, wp, wn,
                                  stream_ptr()))
    return c


# ---- chains batched in lockstep ([B, ...] stacked tensors; every call spans all chains) ----
def _stacked(t: torch.Tensor, name: str, nd: int) -> torch.Tensor:
    t = _f64(t, name)
    if t.ndim != nd:
        raise ValueError(f"{name} must be a stacked [B, ...] tensor with {nd} dimensions (got {tuple(t.shape)})")
    return t


def _bsite_dims(L, W, R):
    B, chi_l, dl, chi_l2 = L.shape
    B2, dl2, dr, d, d2 = W.shape
    B3, chi_r, dr2, chi_r2 = R.shape
    if len({B, B2, B3}) != 1 or chi_l != chi_l2 or chi_r != chi_r2 or dl != dl2 or dr != dr2 or d != d2:
        raise ValueError(f"inconsistent batched L {tuple(L.shape)}, W {tuple(W.shape)}, R {tuple(R.shape)}")
    return B, chi_l, d, chi_r, dl, dr


def batched_matvec1(L, W, R, x, precision="fp64"):
    """y[b] = H_eff[b] x[b] for every chain b (L [B, chi_l, dl, chi_l], W [B, dl, dr, d, d],
    R [B, chi_r, dr, chi_r], x [B, chi_l, d, chi_r])."""
    L, W, R, x = _stacked(L, "L", 4), _stacked(W, "W", 5), _stacked(R, "R", 4), _stacked(x, "x", 4)
    B, chi_l, d, chi_r, dl, dr = _bsite_dims(L, W, R)
    y = torch.empty_like(x)
    wp, wn = Workspace.get(lib.tnx_batched_matvec1_workspace_bytes(chi_l, d, chi_r, dl, dr, B), x.device)
    n = chi_l * d * chi_r
    check("tnx_batched_matvec1", lib.tnx_batched_matvec1(
        ptr(L), chi_l * dl * chi_l, ptr(W), dl * dr * d * d, ptr(R), chi_r * dr * chi_r, ptr(x), n, ptr(y), n, B,
        chi_l, d, chi_r, dl, dr, precision_code(precision), wp, wn, stream_ptr()))
    return y


def batched_full_matrix1(L, W, R):
    L, W, R = _stacked(L, "L", 4), _stacked(W, "W", 5), _stacked(R, "R", 4)
    B, chi_l, d, chi_r, dl, dr = _bsite_dims(L, W, R)
    n = chi_l * d * chi_r
    H = torch.empty((B, n, n), dtype=torch.float64, device=L.device)
    check("tnx_batched_full_matrix1", lib.tnx_batched_full_matrix1(
        ptr(L), chi_l * dl * chi_l, ptr(W), dl * dr * d * d, ptr(R), chi_r * dr * chi_r, ptr(H), B, chi_l, d, chi_r,
        dl, dr, stream_ptr()))
    return H


def batched_env_update(direction: int, E, A, W, precision="fp64"):
    E, A, W = _stacked(E, "E", 4), _stacked(A, "A", 4), _stacked(W, "W", 5)
    B, chi_l, d, chi_r = A.shape
    dl, dr = W.shape[1], W.shape[2]
    if direction == 1:
        if tuple(E.shape) != (B, chi_l, dl, chi_l):
            raise ValueError(f"left environments {tuple(E.shape)} do not match A {tuple(A.shape)} / W")
        shape = (B, chi_r, dr, chi_r)
    elif direction == -1:
        if tuple(E.shape) != (B, chi_r, dr, chi_r):
            raise ValueError(f"right environments {tuple(E.shape)} do not match A {tuple(A.shape)} / W")
        shape = (B, chi_l, dl, chi_l)
    else:
        raise KeyError("direction must be +1 (rightward) or -1 (leftward)")
    out = torch.empty(shape, dtype=torch.float64, device=A.device)
    wp, wn = Workspace.get(lib.tnx_batched_env_update_workspace_bytes(chi_l, d, chi_r, dl, dr, B), A.device)
    check("tnx_batched_env_update", lib.tnx_batched_env_update(
        direction, ptr(E), E[0].numel(), ptr(A), A[0].numel(), ptr(W), W[0].numel(), ptr(out), out[0].numel(), B,
        chi_l, d, chi_r, dl, dr, precision_code(precision), wp, wn, stream_ptr()))
    return out


def batched_davidson1(L, W, R, X, tol=1e-8, max_iter=400, max_basis=24, precision="fp64"):
    """Lowest eigenpair of every chain's H_eff from X[b] (overwritten with the unit Ritz vectors).
    Returns (evals [B], residuals [B], expansions, active mask [B] of chains not converged)."""
    L, W, R = _stacked(L, "L", 4), _stacked(W, "W", 5), _stacked(R, "R", 4)
    if X.dtype != torch.float64 or not X.is_cuda or not X.is_contiguous() or X.ndim != 4:
        raise ValueError("X must be a contiguous float64 CUDA tensor [B, chi_l, d, chi_r] (it is overwritten)")
    B, chi_l, d, chi_r, dl, dr = _bsite_dims(L, W, R)
    n = chi_l * d * chi_r
    evals = torch.empty(B, dtype=torch.float64, device=X.device)
    resid = torch.empty(B, dtype=torch.float64, device=X.device)
    active = torch.empty(B, dtype=torch.int32, device=X.device)
    wp, wn = Workspace.get(lib.tnx_batched_davidson1_workspace_bytes(chi_l, d, chi_r, dl, dr, B, max_basis), X.device)
    it = ctypes.c_int(0)
    st = lib.tnx_batched_davidson1(ptr(L), chi_l * dl * chi_l, ptr(W), dl * dr * d * d, ptr(R), chi_r * dr * chi_r,
                                   ptr(X), n, B, chi_l, d, chi_r, dl, dr, float(tol), int(max_iter), int(max_basis),
                                   precision_code(precision), ptr(evals), ptr(resid), ctypes.byref(it), ptr(active),
                                   wp, wn, stream_ptr())
    if st not in (_lib.TNX_OK, _lib.TNX_ERR_NOT_CONVERGED):
        check("tnx_batched_davidson1", st)
    return evals, resid, it.value, active


def batched_gauge_move(direction: int, a_site: torch.Tensor, a_nb: torch.Tensor, precision="fp64"):
    """In-place gauge move of every chain (QR form of split_tensor) on stacked site tensors."""
    if not (a_site.is_contiguous() and a_nb.is_contiguous()) or a_site.ndim != 4 or a_nb.ndim != 4:
        raise ValueError("stacked MPS tensors [B, chi_l, d, chi_r] must be contiguous")
    B, chi_l, d, chi_r = a_site.shape
    if direction == 1:
        if a_nb.shape[1] != chi_r:
            raise ValueError("right neighbour does not share the bond")
        other = a_nb.shape[3]
    elif direction == -1:
        if a_nb.shape[3] != chi_l:
            raise ValueError("left neighbour does not share the bond")
        other = a_nb.shape[1]
    else:
        raise KeyError("MatrixProductState only supplies left or right direction.")
    wp, wn = Workspace.get(lib.tnx_batched_gauge_move_workspace_bytes(direction, chi_l, d, chi_r, other, B),
                           a_site.device)
    check("tnx_batched_gauge_move", lib.tnx_batched_gauge_move(
        direction, ptr(a_site), a_site[0].numel(), ptr(a_nb), a_nb[0].numel(), B, chi_l, d, chi_r, other,
        precision_code(precision), wp, wn, stream_ptr()))
