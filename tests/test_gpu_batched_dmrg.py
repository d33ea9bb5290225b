"""Independent chains of one shape swept in lockstep (BatchedFiniteDMRG: every kernel spans all
chains), checked kernel by kernel against the oracle and as a whole against per-chain FiniteDMRG
runs and exact diagonalisation; the stream-concurrent form (StreamedFiniteDMRG) for chains of
different shapes."""
import numpy as np
import pytest
import torch

from oracle import ed as oed
from oracle import models as om
from oracle import mps as omps

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _chain_data(B, chi_l, chi_r, seed):
    rng = np.random.RandomState(seed)
    L = rng.standard_normal((B, chi_l, 5, chi_l))
    R = rng.standard_normal((B, chi_r, 5, chi_r))
    L = 0.5 * (L + L.transpose(0, 3, 2, 1))
    R = 0.5 * (R + R.transpose(0, 3, 2, 1))
    W = np.stack([om.uniform(om.random_heisenberg_mpo(6, 1.0, seed=seed + b))[2] for b in range(B)])
    x = rng.standard_normal((B, chi_l, 2, chi_r))
    return L, W, R, x


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_matvec_and_env_update_vs_oracle(cuda, precision):
    import tnpy_gb300.kernels as K

    B, cl, cr = 7, 24, 40
    L, W, R, x = _chain_data(B, cl, cr, 1)
    y = K.batched_matvec1(_t(L, cuda), _t(W, cuda), _t(R, cuda), _t(x, cuda), precision=precision).cpu().numpy()
    A = x  # a site tensor (chi_l, d, chi_r)
    El = K.batched_env_update(1, _t(L, cuda), _t(A, cuda), _t(W, cuda), precision=precision).cpu().numpy()
    Er = K.batched_env_update(-1, _t(R, cuda), _t(A, cuda), _t(W, cuda), precision=precision).cpu().numpy()
    for b in range(B):
        ref = omps.one_site_matvec(L[b], W[b], R[b], x[b])
        np.testing.assert_allclose(y[b], ref, atol=1e-12 * np.abs(ref).max())
        rl = omps.update_left(L[b], A[b], W[b])
        np.testing.assert_allclose(El[b], rl, atol=1e-12 * np.abs(rl).max())
        rr = omps.update_right(R[b], A[b], W[b])
        np.testing.assert_allclose(Er[b], rr, atol=1e-12 * np.abs(rr).max())


@pytest.mark.parametrize("direction", [1, -1])
def test_batched_gauge_move(cuda, direction):
    """Q orthonormal for every chain and the two-site state unchanged; one chain rank deficient."""
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(3)
    B, cl, d, cr, co = 5, 32, 2, 64, 48
    if direction == 1:
        a = rng.standard_normal((B, cl, d, cr))
        nb = rng.standard_normal((B, cr, d, co))
        a[2, :, :, 5:] = 0.0  # rank 5
    else:
        a = rng.standard_normal((B, cl, d, cr))
        nb = rng.standard_normal((B, co, d, cl))
        a[2, 7:] = 0.0
    ta, tn = _t(a, cuda), _t(nb, cuda)
    K.batched_gauge_move(direction, ta, tn)
    qa, qn = ta.cpu().numpy(), tn.cpu().numpy()
    for b in range(B):
        if direction == 1:
            q = qa[b].reshape(cl * d, cr)
            before = np.tensordot(a[b], nb[b], axes=([2], [0]))
            after = np.tensordot(qa[b], qn[b], axes=([2], [0]))
        else:
            q = qa[b].reshape(cl, d * cr).T
            before = np.tensordot(nb[b], a[b], axes=([2], [0]))
            after = np.tensordot(qn[b], qa[b], axes=([2], [0]))
        assert np.abs(q.T @ q - np.eye(q.shape[1])).max() < 1e-12, b
        np.testing.assert_allclose(after, before, atol=1e-12 * np.abs(before).max())


def test_batched_davidson_masks_vs_numpy(cuda):
    """Chains converge after different numbers of expansions; every chain's eigenvalue matches
    its dense spectrum, and no chain is left active."""
    import tnpy_gb300.kernels as K

    B, cl, cr = 6, 8, 8
    # symmetric effective Hamiltonians: environments of random MPSs of random-field chains
    L, W, R = [], [], []
    for b in range(B):
        mpo = om.random_heisenberg_mpo(8, 1.0, seed=20 + b)
        env = omps.Environment(mpo, omps.random_mps(8, 8, 2, seed=30 + b))
        L.append(env.left[4])
        R.append(env.right[4])
        W.append(om.uniform(mpo)[4])
    L, W, R = np.stack(L), np.stack(W), np.stack(R)
    rng = np.random.RandomState(4)
    X = rng.standard_normal((B, cl, 2, cr))
    X[0] = np.linalg.eigh(omps.one_site_full_matrix(L[0], W[0], R[0]))[1][:, 0].reshape(cl, 2, cr)  # converged start
    tX = _t(X, cuda)
    ev, rn, its, active = K.batched_davidson1(_t(L, cuda), _t(W, cuda), _t(R, cuda), tX, tol=1e-10, max_iter=400)
    assert int(active.sum().item()) == 0
    ev = ev.cpu().numpy()
    for b in range(B):
        w = np.linalg.eigvalsh(omps.one_site_full_matrix(L[b], W[b], R[b]))
        assert abs(ev[b] - w[0]) <= 1e-10 * max(1.0, abs(w[0])), (b, ev[b], w[0])
    assert rn.cpu().numpy().max() <= 1e-10 * max(1.0, np.abs(ev).max())
    xb = tX.cpu().numpy().reshape(B, -1)
    np.testing.assert_allclose(np.linalg.norm(xb, axis=1), 1.0, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_chains_match_single_runs(cuda, precision):
    import tnpy_gb300 as tg

    seeds = [100, 101, 102, 103, 104]
    mpos = [tg.model.RandomHeisenberg(16, h=1.0, seed=s).mpo for s in seeds]
    b = tg.BatchedFiniteDMRG(mpos, bond_dim=16, seed=7, precision=precision)
    energies = b.run(tol=1e-10, max_sweep=8)
    assert len(energies) == len(seeds) and b.stats["unconverged"] == 0
    for c, mpo in enumerate(mpos):
        f = tg.FiniteDMRG(mpo, 16, seed=7 + c, compute_variance=False, precision="fp64")
        ref = f.run(tol=1e-10, max_sweep=8)
        assert abs(energies[c][-1] - ref[-1]) <= 1e-9 * abs(ref[-1]), (c, energies[c][-1], ref[-1])


def test_batched_chains_vs_ed(cuda):
    import tnpy_gb300 as tg

    seeds = [100, 101, 102]
    mpos = [om.random_heisenberg_mpo(10, 1.0, seed=s) for s in seeds]
    b = tg.BatchedFiniteDMRG([tg.MatrixProductOperator(m) for m in mpos], chi=32)
    energies = b.run(tol=1e-10, max_sweep=10)
    for m, e in zip(mpos, energies):
        np.testing.assert_allclose(e[-1], oed.ExactDiagonalization(m).evals[0], atol=1e-8)
    assert all(1 <= s <= 10 for s in b.sweeps)
    # a chain's state is its own: <H> of chain 1's MPS under chain 1's MPO is its energy
    from tnpy_gb300.matrix_product_state import expectation_value

    m1 = b.mps(1)
    e1 = expectation_value(m1, tg.MatrixProductOperator(mpos[1])) / expectation_value(m1)
    np.testing.assert_allclose(e1, energies[1][-1], atol=1e-8)


def test_batched_needs_one_shape(cuda):
    import tnpy_gb300 as tg

    with pytest.raises(ValueError):
        tg.BatchedFiniteDMRG([], bond_dim=8)
    with pytest.raises(ValueError):
        tg.BatchedFiniteDMRG([tg.model.XXZ(8, 0.5).mpo, tg.model.XXZ(10, 0.5).mpo], bond_dim=8)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_streamed_chains_equal_single_runs(cuda, precision):
    import tnpy_gb300 as tg

    seeds = [100, 101, 102, 103, 104]
    mpos = [tg.model.RandomHeisenberg(16, h=1.0, seed=s).mpo for s in seeds]
    b = tg.StreamedFiniteDMRG(mpos, bond_dim=16, workers=3, seed=7, compute_variance=False, precision=precision)
    energies = b.run(tol=1e-10, max_sweep=6)
    assert len(energies) == len(seeds)
    for c, mpo in enumerate(mpos):
        f = tg.FiniteDMRG(mpo, 16, seed=7, compute_variance=False, precision=precision)
        ref = f.run(tol=1e-10, max_sweep=6)
        # same kernels, fixed reduction orders: the stream a chain runs on does not change its arithmetic
        assert energies[c] == pytest.approx(ref, abs=1e-12, rel=0), (c, energies[c], ref)
