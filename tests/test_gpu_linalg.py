"""tnpy.linalg call shapes on the device (tnpy/linalg.py:9-87) and the Schmidt values of an MPS
bond: the one-sided Jacobi SVD against np.linalg.svd (graded spectra down to 1e-12, rank
deficiency, wide and tall shapes), the truncated QR, eigshmv on a one-site operator, and the
entanglement spectrum of a DMRG ground state against the oracle's full state vector."""
import numpy as np
import pytest
import torch

from oracle import dmrg as odmrg
from oracle import models as om
from oracle import mps as omps

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _orth_err(q):
    return np.abs(q.T @ q - np.eye(q.shape[1])).max()


@pytest.mark.parametrize("m,n", [(1, 1), (5, 3), (7, 7), (64, 64), (300, 128), (513, 257), (1024, 1024)])
def test_svd_jacobi_matches_numpy(cuda, m, n):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(m * 7 + n)
    a = rng.standard_normal((m, n))
    u, s, vt = (x.cpu().numpy() for x in K.svd(_t(a, cuda)))
    s_ref = np.linalg.svd(a, compute_uv=False)
    # both SVDs are backward stable: absolute agreement at a modest multiple of eps * s_max
    # (measured 1.6e-13 s_max at 1024 x 1024, where each column takes ~10^4 rotations)
    assert np.abs(s - s_ref).max() <= 1e-12 * s_ref[0], np.abs(s - s_ref).max()
    assert _orth_err(u) < 1e-12 and _orth_err(vt.T) < 1e-12
    assert np.abs(u @ np.diag(s) @ vt - a).max() < 1e-12 * s_ref[0]


def test_svd_graded_spectrum_down_to_1e_12(cuda):
    import tnpy_gb300.linalg as la

    rng = np.random.RandomState(5)
    n = 200
    s_true = np.logspace(0, -12, n)
    u0, _ = np.linalg.qr(rng.standard_normal((2 * n, n)))
    v0, _ = np.linalg.qr(rng.standard_normal((n, n)))
    a = (u0 * s_true) @ v0.T
    u, s, vt = (x.cpu().numpy() for x in la.svd(a, cutoff=n))
    s_np = np.linalg.svd(a, compute_uv=False)
    # both decompositions are backward stable: absolute agreement at a few hundred eps * s_max
    # (measured 4.2e-14); a Gram-matrix route would leave ~1e-8 on the small values
    assert np.abs(s - s_np).max() < 2e-13, np.abs(s - s_np).max()
    assert np.abs(s - s_true).max() < 2e-13
    # the Schmidt-like tail keeps its leading digits down to 1e-8 * s_max (a Gram matrix would not)
    tail = s_true > 1e-8
    assert np.abs(s[tail] / s_true[tail] - 1).max() < 2e-5
    assert _orth_err(u) < 1e-12 and _orth_err(vt.T) < 1e-12


def test_svd_rank_deficient(cuda):
    import tnpy_gb300.linalg as la

    rng = np.random.RandomState(11)
    a = rng.standard_normal((40, 6)) @ rng.standard_normal((6, 24))  # rank 6
    a[:, 3] = 0.0  # an exactly zero column as well
    u, s, vt = (x.cpu().numpy() for x in la.svd(a, cutoff=24))
    s_np = np.linalg.svd(a, compute_uv=False)
    assert np.abs(s - s_np).max() < 1e-13 * s_np[0]
    assert np.all(s[6:] < 1e-13 * s[0])
    assert _orth_err(u) < 1e-12 and _orth_err(vt.T) < 1e-12
    assert np.abs(u @ np.diag(s) @ vt - a).max() < 1e-12 * s_np[0]


def test_svd_wide_and_cutoff(cuda):
    import tnpy_gb300.linalg as la

    rng = np.random.RandomState(2)
    a = rng.standard_normal((20, 50))
    u, s, vt = la.svd(a, cutoff=8)
    assert tuple(u.shape) == (20, 8) and tuple(s.shape) == (8,) and tuple(vt.shape) == (8, 50)
    s_np = np.linalg.svd(a, compute_uv=False)
    np.testing.assert_allclose(s.cpu().numpy(), s_np[:8], rtol=1e-13)


@pytest.mark.parametrize("m,n,cutoff", [(30, 12, 12), (30, 12, 5), (12, 30, 7), (64, 64, 64)])
def test_qr_cutoff_shapes_and_factors(cuda, m, n, cutoff):
    """linalg.qr(matrix, cutoff) = the reduced QR sliced to cutoff (tnpy/linalg.py:26-39)."""
    import tnpy_gb300.linalg as la

    rng = np.random.RandomState(m + n + cutoff)
    a = rng.standard_normal((m, n))
    q, r = (x.cpu().numpy() for x in la.qr(a, cutoff))
    q_ref, r_ref = omps.qr(a, cutoff)
    assert q.shape == q_ref.shape and r.shape == r_ref.shape
    assert _orth_err(q) < 1e-12
    # the same factors up to column signs
    sg = np.sign(np.diag(r[:, :min(cutoff, n)])) * np.sign(np.diag(r_ref[:, :min(cutoff, n)]))
    np.testing.assert_allclose(q * sg[None, :], q_ref, atol=1e-12)
    np.testing.assert_allclose(r * sg[:, None], r_ref, atol=1e-12 * np.abs(a).max() * np.sqrt(m))
    if cutoff >= min(m, n):
        np.testing.assert_allclose(q @ r, a, atol=1e-12 * np.abs(a).max() * np.sqrt(m))


def test_eigshmv_on_one_site_operator(cuda):
    """linalg.eigshmv(Environment.one_site_matvec(site), v0) -> (float, (N, 1)) (tnpy/linalg.py:64-87)."""
    import tnpy_gb300 as tg
    import tnpy_gb300.linalg as la

    mps = tg.MatrixProductState.random(10, 16, 2, seed=4)
    env = tg.Environment(tg.model.XXZ(10, -0.5).mpo, mps)
    site = 5
    op = env.one_site_matvec(site)
    e, v = la.eigshmv(op, mps[site].reshape(-1, 1), tol=1e-12)
    n = mps.tensors[site].numel()
    assert isinstance(e, float) and tuple(v.shape) == (n, 1)
    L, W, R = (t.cpu().numpy() for t in env.site_operator(site))
    w = np.linalg.eigvalsh(omps.one_site_full_matrix(L, W, R))
    assert abs(e - w[0]) < 1e-11 * abs(w[0])
    hv = op.matvec(v)
    assert torch.linalg.vector_norm(hv - e * v).item() < 1e-9 * abs(e)
    with pytest.raises(NotImplementedError):
        la.eigshmv(op, mps[site].reshape(-1, 1), k=2)


def _state_vector(mps):
    psi = mps[0]
    for a in mps[1:]:
        psi = np.tensordot(psi, a, axes=([-1], [0]))
    return psi.reshape(-1)


@pytest.mark.parametrize("bond", [2, 5, 8])
def test_entanglement_spectrum_matches_full_state(cuda, bond):
    """Schmidt values of a converged fDMRG state (XXZ(12, -0.5), chi=16) against the SVD of the
    oracle's full state vector reshaped at the bond."""
    import tnpy_gb300 as tg

    n = 12
    f = tg.FiniteDMRG(tg.MatrixProductOperator(om.xxz_mpo(n, -0.5)), bond_dim=16, seed=7, compute_variance=False)
    f.run(tol=1e-10, max_sweep=8)
    lam = f.measurements.entanglement_spectrum(bond)
    psi = _state_vector([t.cpu().numpy() for t in f.mps.tensors])
    psi /= np.linalg.norm(psi)
    s_ref = np.linalg.svd(psi.reshape(2 ** (bond + 1), -1), compute_uv=False)
    k = lam.size
    assert abs(np.sum(lam**2) - 1) < 1e-12
    np.testing.assert_allclose(lam, s_ref[:k], atol=1e-12)
    # the spectrum of a gauge-moved copy is the same state's: nothing in f.mps changed
    lam2 = f.measurements.entanglement_spectrum(bond)
    np.testing.assert_array_equal(lam, lam2)


def test_entanglement_spectrum_of_oracle_dmrg_state(cuda):
    """The same reporting on a state produced by the oracle's own fDMRG (loaded into the device
    MPS): the spectra of the two implementations' ground states agree at 1e-8."""
    import tnpy_gb300 as tg

    n, chi = 14, 24
    mpo = om.xxz_mpo(n, -0.5)
    o = odmrg.FiniteDMRG(mpo, chi=chi, seed=3)
    o.run(tol=1e-11, max_sweep=10, with_variance=False)
    f = tg.FiniteDMRG(tg.MatrixProductOperator(mpo), bond_dim=chi, seed=3, compute_variance=False)
    f.run(tol=1e-11, max_sweep=10)
    lam_gpu = f.measurements.entanglement_spectrum(n // 2 - 1)
    lam_ora = tg.MatrixProductStateMeasurements(tg.MatrixProductState(o.mps, device=cuda)).entanglement_spectrum(
        n // 2 - 1)
    np.testing.assert_allclose(lam_gpu, lam_ora, atol=1e-8)
