"""Parity of the CUDA kernels (through the C ABI) against the CPU oracle."""
import numpy as np
import pytest
import torch

from oracle import models as om
from oracle import mps as omps

pytestmark = pytest.mark.gpu


def _rand_env(chi_l, chi_r, dl, dr, d=2, seed=0, sym=True):
    rng = np.random.RandomState(seed)
    L = rng.standard_normal((chi_l, dl, chi_l))
    R = rng.standard_normal((chi_r, dr, chi_r))
    if sym:  # environments of a Hermitian MPO are symmetric in (ket, bra)
        L = 0.5 * (L + L.transpose(2, 1, 0))
        R = 0.5 * (R + R.transpose(2, 1, 0))
    W = rng.standard_normal((dl, dr, d, d))
    W = 0.5 * (W + W.transpose(0, 1, 3, 2))
    x = rng.standard_normal((chi_l, d, chi_r))
    return L, W, R, x


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("chi_l,chi_r,dl,dr", [(1, 2, 1, 5), (4, 8, 5, 5), (37, 29, 5, 5), (64, 64, 5, 5),
                                               (130, 96, 5, 5), (256, 256, 5, 5), (16, 1, 5, 1), (12, 12, 25, 25)])
def test_matvec1_fp64(cuda, chi_l, chi_r, dl, dr):
    import tnpy_gb300.kernels as K

    L, W, R, x = _rand_env(chi_l, chi_r, dl, dr, seed=chi_l + chi_r)
    y = K.matvec1(_t(L, cuda), _t(W, cuda), _t(R, cuda), _t(x, cuda)).cpu().numpy()
    y_ref = omps.one_site_matvec(L, W, R, x)
    np.testing.assert_allclose(y, y_ref, rtol=1e-12, atol=1e-12 * np.abs(y_ref).max())


@pytest.mark.parametrize("chi_l,chi_r,dl,dr", [(1, 2, 1, 5), (8, 16, 5, 5), (33, 47, 5, 5), (128, 128, 5, 5)])
def test_env_update_fp64(cuda, chi_l, chi_r, dl, dr):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(chi_l * 7 + chi_r)
    A = rng.standard_normal((chi_l, 2, chi_r))
    W = rng.standard_normal((dl, dr, 2, 2))
    L = rng.standard_normal((chi_l, dl, chi_l))
    R = rng.standard_normal((chi_r, dr, chi_r))
    out = K.env_update(1, _t(L, cuda), _t(A, cuda), _t(W, cuda)).cpu().numpy()
    ref = omps.update_left(L, A, W)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    out = K.env_update(-1, _t(R, cuda), _t(A, cuda), _t(W, cuda)).cpu().numpy()
    ref = omps.update_right(R, A, W)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_full_matrix_and_diag(cuda):
    import tnpy_gb300.kernels as K

    L, W, R, _ = _rand_env(6, 5, 5, 5, seed=3)
    H = K.full_matrix1(_t(L, cuda), _t(W, cuda), _t(R, cuda)).cpu().numpy()
    np.testing.assert_allclose(H, omps.one_site_full_matrix(L, W, R), atol=1e-12)
    D = K.diag1(_t(L, cuda), _t(W, cuda), _t(R, cuda)).cpu().numpy()
    np.testing.assert_allclose(D, omps.one_site_diagonal(L, W, R), atol=1e-12)


@pytest.mark.parametrize("sizes,keep", [([4], 4), ([1, 2, 3], 1), ([16, 31, 64], 3), ([199], 1), ([128, 100], 32)])
def test_eigh_batched(cuda, sizes, keep):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(sum(sizes))
    mats = []
    for s in sizes:
        a = rng.standard_normal((s, s))
        mats.append(a + a.T)
    ev, vec = K.eigh_batched([_t(m, cuda) for m in mats], keep=keep)
    ev, vec = ev.cpu().numpy(), vec.cpu().numpy()
    for b, m in enumerate(mats):
        w, v = np.linalg.eigh(m)
        np.testing.assert_allclose(ev[b], w[:keep], atol=1e-12 * np.abs(w).max())
        for j in range(keep):
            vj = vec[b, : m.shape[0], j]
            np.testing.assert_allclose(abs(vj @ v[:, j]), 1.0, atol=1e-10)
            np.testing.assert_allclose(m @ vj, w[j] * vj, atol=1e-11 * np.abs(w).max())


def test_eigh_degenerate_kat(cuda, golden):
    """tests/test_exact_diagonalization.py:10-42 of the reference: n=2 Heisenberg spectrum."""
    import tnpy_gb300 as tg

    h = np.array(golden["ed_n2"]["matrix"])
    ev, vec = tg.linalg.eigh(h, k=4)
    np.testing.assert_allclose(ev.cpu().numpy(), golden["ed_n2"]["evals"], atol=1e-15)
    v = vec.cpu().numpy()
    np.testing.assert_allclose(v.T @ v, np.eye(4), atol=1e-14)


@pytest.mark.parametrize("m,n", [(4, 4), (64, 32), (100, 37), (512, 256), (2048, 1024), (300, 300)])
def test_qr(cuda, m, n):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(m + n)
    a = rng.standard_normal((m, n))
    q, r = K.qr(_t(a, cuda))
    q, r = q.cpu().numpy(), r.cpu().numpy()
    np.testing.assert_allclose(q.T @ q, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(q @ r, a, atol=1e-12 * np.abs(a).max() * np.sqrt(n))
    assert np.allclose(np.tril(r, -1), 0)


@pytest.mark.parametrize("m,n", [(300, 300), (1100, 700)])
def test_qr_stale_workspace(cuda, m, n):
    """The QR reads no scratch it has not written: the workspace is filled with NaN first
    (two outer blocks of 256 columns and a ragged third / a ragged second)."""
    import tnpy_gb300.kernels as K
    from tnpy_gb300._lib import lib

    rng = np.random.RandomState(7)
    a = rng.standard_normal((m, n))
    _poison_workspace(lib.tnx_qr_workspace_bytes(m, n), cuda)
    q, r = K.qr(_t(a, cuda))
    q, r = q.cpu().numpy(), r.cpu().numpy()
    np.testing.assert_allclose(q.T @ q, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(q @ r, a, atol=1e-12 * np.abs(a).max() * np.sqrt(n))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gauge_move_stale_workspace(cuda, precision):
    """Gauge move (chi 600 x 2 x 600 site, both directions) on a NaN-filled workspace."""
    import tnpy_gb300.kernels as K
    from tnpy_gb300._lib import lib

    rng = np.random.RandomState(5)
    chi = 600
    for direction in (1, -1):
        a = rng.standard_normal((chi, 2, chi))
        nbr = rng.standard_normal((chi, 2, 8)) if direction == 1 else rng.standard_normal((8, 2, chi))
        ta, tn = _t(a, cuda), _t(nbr, cuda)
        _poison_workspace(lib.tnx_gauge_move_workspace_bytes(direction, chi, 2, chi, 8), cuda)
        K.gauge_move(direction, ta, tn, precision=precision)
        q = ta.cpu().numpy().reshape(chi * 2, chi) if direction == 1 else ta.cpu().numpy().reshape(chi, 2 * chi).T
        np.testing.assert_allclose(q.T @ q, np.eye(chi), atol=1e-12)
        # the two-site contraction is unchanged by the move
        before = np.tensordot(a, nbr, axes=([2], [0])) if direction == 1 else np.tensordot(nbr, a, axes=([2], [0]))
        after = (np.tensordot(ta.cpu().numpy(), tn.cpu().numpy(), axes=([2], [0])) if direction == 1
                 else np.tensordot(tn.cpu().numpy(), ta.cpu().numpy(), axes=([2], [0])))
        np.testing.assert_allclose(after, before, atol=1e-11 * np.abs(before).max())


def _poison_workspace(nbytes, device):
    """Fill the library's scratch buffer for the current stream with 0xFF bytes (NaN doubles)."""
    import torch

    from tnpy_gb300._lib import Workspace

    Workspace.get(nbytes, device)
    idx = device.index if device.index is not None else torch.cuda.current_device()
    Workspace._bufs[(idx, torch.cuda.current_stream(idx).cuda_stream)].fill_(255)


def test_qr_rank_deficient(cuda):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(1)
    a = rng.standard_normal((80, 5)) @ rng.standard_normal((5, 40))  # rank 5
    a[:, 7] = 0.0
    q, r = K.qr(_t(a, cuda))
    q, r = q.cpu().numpy(), r.cpu().numpy()
    np.testing.assert_allclose(q.T @ q, np.eye(40), atol=1e-13)
    np.testing.assert_allclose(q @ r, a, atol=1e-12 * np.abs(a).max() * 10)


@pytest.mark.parametrize("direction", [1, -1])
def test_gauge_move(cuda, direction):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(7)
    a = rng.standard_normal((16, 2, 32))
    if direction == 1:
        nb = rng.standard_normal((32, 2, 24))
        two = np.tensordot(a, nb, axes=([2], [0]))
    else:
        a = rng.standard_normal((32, 2, 16))
        nb = rng.standard_normal((24, 2, 32))
        two = np.tensordot(nb, a, axes=([2], [0]))
    ta, tn = _t(a, cuda), _t(nb, cuda)
    K.gauge_move(direction, ta, tn)
    a2, nb2 = ta.cpu().numpy(), tn.cpu().numpy()
    if direction == 1:
        m = a2.reshape(-1, a2.shape[2])
        np.testing.assert_allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-13)
        np.testing.assert_allclose(np.tensordot(a2, nb2, axes=([2], [0])), two, atol=1e-12)
    else:
        m = a2.reshape(a2.shape[0], -1)
        np.testing.assert_allclose(m @ m.T, np.eye(m.shape[0]), atol=1e-13)
        np.testing.assert_allclose(np.tensordot(nb2, a2, axes=([2], [0])), two, atol=1e-12)


@pytest.mark.parametrize("chi", [8, 24, 64])
def test_davidson_lowest_eigenpair(cuda, chi):
    import tnpy_gb300.kernels as K

    mpo = om.uniform(om.xxz_mpo(12, -0.5))
    m = omps.random_mps(12, chi, 2, seed=chi)
    env = omps.Environment(om.xxz_mpo(12, -0.5), m)
    site = 6
    L, W, R = env.left[site], mpo[site], env.right[site]
    H = omps.one_site_full_matrix(L, W, R)
    w, v = np.linalg.eigh(H)
    x = _t(m[site], cuda).clone()
    e, rn, its, ok = K.davidson1(_t(L, cuda), _t(W, cuda), _t(R, cuda), x, tol=1e-10, max_iter=500)
    assert ok, (rn, its)
    np.testing.assert_allclose(e, w[0], atol=1e-11 * abs(w[0]))
    xv = x.cpu().numpy().reshape(-1)
    assert abs(abs(xv @ v[:, 0]) - 1) < 1e-9


def test_split_tensor_invariance_device(cuda):
    """tests/test_matrix_product_state.py:83-89 of the reference, on the device."""
    import tnpy_gb300 as tg

    mps = tg.MatrixProductState.random(8, 10, 2, seed=5)
    for site in (2, 3, 4, 6):
        two = torch.tensordot(mps.tensors[site], mps.tensors[site + 1], dims=([2], [0])).cpu().numpy()
        mps.split_tensor(site, tg.Direction.RIGHTWARD)
        after = torch.tensordot(mps.tensors[site], mps.tensors[site + 1], dims=([2], [0])).cpu().numpy()
        np.testing.assert_allclose(after, two, atol=1e-12)


def test_random_mps_shapes(cuda):
    """tests/test_matrix_product_state.py:11-49 of the reference."""
    import tnpy_gb300 as tg

    mps = tg.MatrixProductState.random(n=8, bond_dim=10, phys_dim=2)
    assert tuple(mps[0].shape) == (2, 2)
    assert tuple(mps[1].shape) == (2, 2, 4)
    assert tuple(mps[2].shape) == (4, 2, 8)
    assert tuple(mps[-2].shape) == (4, 2, 2)
    assert tuple(mps[-1].shape) == (2, 2)
    np.testing.assert_allclose(tg.matrix_product_state.expectation_value(mps), 1.0, atol=1e-12)
    ref = omps.random_mps(8, 10, 2, seed=1234)
    # same seeded tensors before canonicalisation -> same state up to gauge: compare norms of
    # the contracted states
    psi = ref[0]
    for a in ref[1:]:
        psi = np.tensordot(psi, a, axes=([-1], [0]))
    got = mps.tensors[0].cpu().numpy()
    for a in mps.tensors[1:]:
        got = np.tensordot(got, a.cpu().numpy(), axes=([-1], [0]))
    np.testing.assert_allclose(abs(psi.reshape(-1) @ got.reshape(-1)), 1.0, atol=1e-12)


@pytest.mark.parametrize("m,n,k,ta,tb", [(64, 128, 16, False, False), (300, 260, 1000, True, False),
                                         (1024, 37, 513, False, True), (5, 3, 7, True, True)])
def test_gemm_df64(cuda, m, n, k, ta, tb):
    """Double-FP32 GEMM: FP64-class accuracy (~2^-48 per product)."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(m + k)
    a = rng.standard_normal((k, m) if ta else (m, k))
    b = rng.standard_normal((n, k) if tb else (k, n))
    c = K.gemm_df64(_t(a, cuda), _t(b, cuda), trans_a=ta, trans_b=tb).cpu().numpy()
    ref = (a.T if ta else a) @ (b.T if tb else b)
    scale = np.abs(a).max() * np.abs(b).max() * k
    assert np.abs(c - ref).max() <= 1e-13 * scale, np.abs(c - ref).max() / scale


@pytest.mark.parametrize("chi_l,chi_r", [(8, 16), (64, 64), (130, 96)])
def test_env_update_df64(cuda, chi_l, chi_r):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(chi_l)
    A = rng.standard_normal((chi_l, 2, chi_r))
    W = rng.standard_normal((5, 5, 2, 2))
    L = rng.standard_normal((chi_l, 5, chi_l))
    R = rng.standard_normal((chi_r, 5, chi_r))
    for direction, E, ref in ((1, L, omps.update_left(L, A, W)), (-1, R, omps.update_right(R, A, W))):
        out = K.env_update(direction, _t(E, cuda), _t(A, cuda), _t(W, cuda), precision="df64").cpu().numpy()
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_gauge_move_df64(cuda):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(11)
    a = rng.standard_normal((64, 2, 128))
    nb = rng.standard_normal((128, 2, 40))
    two = np.tensordot(a, nb, axes=([2], [0]))
    ta, tn = _t(a, cuda), _t(nb, cuda)
    K.gauge_move(1, ta, tn, precision="mixed")
    a2, nb2 = ta.cpu().numpy(), tn.cpu().numpy()
    m = a2.reshape(-1, 128)
    np.testing.assert_allclose(m.T @ m, np.eye(128), atol=1e-12)
    np.testing.assert_allclose(np.tensordot(a2, nb2, axes=([2], [0])), two, atol=1e-11)


@pytest.mark.parametrize("chi", [512, 1024])
@pytest.mark.parametrize("direction", [1, -1])
def test_gauge_move_df64_rank_deficient(cuda, direction, chi):
    """chi=512 and 1024 gauge moves in the FP64-class form (double-FP32 panels, Q from the
    compact WY form on the tensor cores) on a site tensor whose Schmidt values span 20 decades,
    as converged MPS bonds do: Q stays orthonormal to 1e-12 and the two-site product is
    reproduced to 1e-11 of its norm."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(5)
    d = 2
    if direction == 1:
        m, n = chi * d, chi
    else:
        m, n = chi * d, chi
    u, _ = np.linalg.qr(rng.standard_normal((m, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = 10.0 ** (-np.linspace(0, 20, n))
    psi = (u * s) @ v.T  # m x n, numerically rank deficient
    if direction == 1:
        a = psi.reshape(chi, d, chi)
        nb = rng.standard_normal((chi, d, 64))
        two = np.tensordot(a, nb, axes=([2], [0]))
    else:
        a = psi.T.reshape(chi, d, chi)  # (chi_l) x (d chi_r)
        nb = rng.standard_normal((64, d, chi))
        two = np.tensordot(nb, a, axes=([2], [0]))
    ta, tn = _t(a, cuda), _t(nb, cuda)
    K.gauge_move(direction, ta, tn, precision="mixed")
    a2, nb2 = ta.cpu().numpy(), tn.cpu().numpy()
    if direction == 1:
        q = a2.reshape(-1, chi)
        np.testing.assert_allclose(q.T @ q, np.eye(chi), atol=1e-12)
        back = np.tensordot(a2, nb2, axes=([2], [0]))
    else:
        q = a2.reshape(chi, -1)
        np.testing.assert_allclose(q @ q.T, np.eye(chi), atol=1e-12)
        back = np.tensordot(nb2, a2, axes=([2], [0]))
    assert np.max(np.abs(back - two)) <= 1e-11 * np.max(np.abs(two))


def test_gemm_oz_nonfinite_propagates(cuda):
    """A row of op(A) or a column of op(B) holding Inf / NaN gives NaN outputs (its integer slices
    are not the value); every other output is the ordinary FP64-class product."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(17)
    a, b = rng.standard_normal((300, 200)), rng.standard_normal((200, 150))
    a[3, 5], a[7, 0], b[9, 11] = np.nan, np.inf, -np.inf
    got = K.gemm_oz(_t(a, cuda), _t(b, cuda)).cpu().numpy()
    bad_rows, bad_cols = [3, 7], [11]
    assert np.isnan(got[bad_rows]).all() and np.isnan(got[:, bad_cols]).all()
    keep_r = np.setdiff1d(np.arange(300), bad_rows)
    keep_c = np.setdiff1d(np.arange(150), bad_cols)
    ok = np.ix_(keep_r, keep_c)
    ref = a[keep_r] @ b[:, keep_c]
    bound = np.abs(a[keep_r]) @ np.abs(b[:, keep_c])
    assert np.max(np.abs(got[ok] - ref) / bound) < 1e-13


def test_gauge_move_mixed_propagates_nan(cuda):
    """A NaN in the site tensor reaches Q and the neighbour in the FP64-class form, as it does in
    FP64 arithmetic (numpy's QR), instead of being flushed to a finite value."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(23)
    a = rng.standard_normal((64, 2, 128))
    a[10, 1, 5] = np.nan
    nb = rng.standard_normal((128, 2, 40))
    ta, tn = _t(a, cuda), _t(nb, cuda)
    K.gauge_move(1, ta, tn, precision="mixed")
    assert np.isnan(ta.cpu().numpy()).any() and np.isnan(tn.cpu().numpy()).any()


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("m,n,k", [(128, 64, 128), (300, 200, 500), (1000, 130, 1024), (5, 7, 3), (257, 65, 1500)])
def test_gemm_oz(cuda, ta, tb, m, n, k):
    """Ozaki-sliced tensor-core GEMM against the FP64 product on N(0,1) operands: error below
    1e-13 of sum_k |a_ik| |b_kj|."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(m + n + k)
    a = rng.standard_normal((k, m) if ta else (m, k))
    b = rng.standard_normal((n, k) if tb else (k, n))
    opa, opb = (a.T if ta else a), (b.T if tb else b)
    ref = opa @ opb
    bound = np.abs(opa) @ np.abs(opb)
    got = K.gemm_oz(_t(a, cuda), _t(b, cuda), trans_a=ta, trans_b=tb).cpu().numpy()
    assert np.max(np.abs(got - ref) / bound) < 1e-13


def test_gemm_oz_wide_range(cuda):
    """Entries spanning ~20 decades: the slicing error is relative to each row's and column's
    maximum, so the error is bounded by 1e-14 K max|a_i.| max|b_.j|."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(8)
    m, n, k = 384, 192, 768
    a = rng.standard_normal((m, k)) * 10.0 ** rng.uniform(-10, 10, (m, k))
    b = rng.standard_normal((k, n)) * 10.0 ** rng.uniform(-10, 10, (k, n))
    got = K.gemm_oz(_t(a, cuda), _t(b, cuda)).cpu().numpy()
    bound = k * np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :]
    assert np.max(np.abs(got - a @ b) / bound) < 1e-14


def test_gemm_oz_exact_small_integers(cuda):
    """Integer operands below 2^7 make every slice exact: the product is bit-exact."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(3)
    a = rng.randint(-100, 100, (256, 640)).astype(np.float64)
    b = rng.randint(-100, 100, (640, 192)).astype(np.float64)
    got = K.gemm_oz(_t(a, cuda), _t(b, cuda)).cpu().numpy()
    np.testing.assert_array_equal(got, a @ b)


@pytest.mark.parametrize("nsplit", [1, 3, 16])
def test_gemm_oz_batched_split_and_mask(cuda, nsplit):
    """Batched tensor-core FP64-class products (one launch over 5 operand sets, K split into
    `nsplit` ranges summed in order) against numpy, within the Ozaki bound 1e-13 of |A||B|; the
    set masked out keeps its previous C."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(31)
    a = rng.standard_normal((5, 150, 700))
    b = rng.standard_normal((5, 700, 90)) * np.logspace(-8, 3, 90)[None, None, :]
    c0 = rng.standard_normal((5, 150, 90))
    mask = np.array([1, 1, 0, 1, 1], dtype=np.int32)
    out = K.gemm_oz_batched(_t(a, cuda), _t(b, cuda), _t(c0.copy(), cuda), alpha=0.5, beta=2.0, nsplit=nsplit,
                            mask=torch.from_numpy(mask)).cpu().numpy()
    for i in range(5):
        if mask[i]:
            ref = 0.5 * a[i] @ b[i] + 2.0 * c0[i]
            bound = 0.5 * np.abs(a[i]) @ np.abs(b[i]) + 2.0 * np.abs(c0[i])
            assert np.max(np.abs(out[i] - ref) / bound) < 1e-13, i
        else:
            np.testing.assert_array_equal(out[i], c0[i])


@pytest.mark.parametrize("sizes,keep", [([4], 4), ([1, 2, 3], 1), ([16, 31, 64], 3), ([64, 64, 40], 32)])
def test_eigh_batched_df64(cuda, sizes, keep):
    """Double-FP32 Jacobi (matrices up to 64 rows) against numpy: eigenvalues to 1e-13 of the
    spectral radius, eigenvectors to 1e-11 in the residual, including a matrix with a
    degenerate cluster."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(7 + sum(sizes))
    mats = []
    for i, s in enumerate(sizes):
        a = rng.standard_normal((s, s))
        a = a + a.T
        if i == 0 and s >= 4:  # a degenerate pair: two equal eigenvalues
            w, v = np.linalg.eigh(a)
            w[1] = w[0]
            a = (v * w) @ v.T
            a = 0.5 * (a + a.T)
        mats.append(a)
    ev, vec = K.eigh_batched([_t(m, cuda) for m in mats], keep=keep, precision="df64")
    ev, vec = ev.cpu().numpy(), vec.cpu().numpy()
    for b, m in enumerate(mats):
        w, _ = np.linalg.eigh(m)
        k = min(keep, m.shape[0])
        np.testing.assert_allclose(ev[b, :k], w[:k], atol=1e-13 * np.abs(w).max())
        v = vec[b, : m.shape[0], :k]
        np.testing.assert_allclose(v.T @ v, np.eye(k), atol=1e-12)
        np.testing.assert_allclose(m @ v, v * ev[b, :k], atol=1e-11 * np.abs(w).max())
