"""Shift-invert DMRG (tnpy/finite_dmrg.py:266-407) on the device, following the reference's own
test class (tests/test_finite_dmrg.py:26-75): RandomHeisenberg(n=10, h=10.5, seed=2022),
bond_dim=64, offsets -0.1, 0.1, 0.2; the energy is the exact eigenvalue nearest below the offset
(1e-6 there; checked here at 1e-9), the restored state its eigenvector up to sign, and the
restored state's <H> that energy. Also the generalised Davidson against the dense pencil and the
MPO application against the oracle."""
import numpy as np
import pytest
import scipy.linalg as spl
import torch

from oracle import dmrg as odmrg
from oracle import models as om
from oracle import mps as omps
from oracle import operators as oops

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_gdavidson_vs_dense_generalised(cuda, precision):
    import tnpy_gb300.kernels as K

    n, eps = 10, -1.3
    arr = om.random_heisenberg_mpo(n, 0.5, offset=eps, seed=3)
    sq = oops.mpo_square(arr)
    mps = omps.random_mps(n, 8, 2, seed=4)
    env, env2 = omps.Environment(arr, mps), omps.Environment(sq, mps)
    site = 5
    ops = (env.left[site], om.uniform(arr)[site], env.right[site], env2.left[site], om.uniform(sq)[site],
           env2.right[site])
    A = omps.one_site_full_matrix(*ops[:3])
    B = omps.one_site_full_matrix(*ops[3:])
    w = spl.eigh(A, b=B, eigvals_only=True)
    x = _t(mps[site], cuda).clone()
    e, rn, its, ok = K.gdavidson1(*(_t(a, cuda) for a in ops), x, tol=1e-10, max_basis=48, precision=precision)
    # this pencil converges slowly near its floor: accepted there (stagnation below 1e-6 |lambda|)
    assert ok, (e, rn, its)
    assert rn <= 1e-6 * max(1.0, abs(e))
    assert abs(e - w[0]) <= 1e-10 * max(1.0, abs(w[0])), (e, w[0])
    xv = x.cpu().numpy().reshape(-1)
    assert abs(xv @ B @ xv - 1.0) < 1e-10


def test_mpo_apply_site_vs_oracle(cuda):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(1)
    a = rng.standard_normal((6, 2, 5))
    w = rng.standard_normal((3, 4, 2, 2))
    out = K.mpo_apply_site(_t(a, cuda), _t(w, cuda)).cpu().numpy()
    t = np.einsum("wvkb,abc->awkcv", w, a)
    ref = t.reshape(6 * 3, 2, 5 * 4)
    np.testing.assert_allclose(out, ref, atol=1e-13)


@pytest.fixture(scope="module")
def ed_system():
    base = om.random_heisenberg_mpo(10, 10.5, seed=2022)
    w, V = np.linalg.eigh(oops.full_hamiltonian(base))
    return base, w, V


@pytest.mark.parametrize("offset", [-0.1, 0.1, 0.2])
def test_shift_invert_dmrg_vs_ed_and_oracle(cuda, ed_system, offset):
    import tnpy_gb300 as tg
    from tnpy_gb300.matrix_product_state import expectation_value

    base, w, V = ed_system
    arr = om.random_heisenberg_mpo(10, 10.5, offset=offset, seed=2022)
    f = tg.ShiftInvertDMRG(tg.MatrixProductOperator(arr), bond_dim=64, offset=offset, seed=5)
    e = f.run(tol=1e-8, max_sweep=20)
    idx = np.where(w < offset)[0][np.argmax(w[w < offset])]
    # local pencils near the shift converge slowly: some sites may stop at max_iter with the
    # Ritz pair already accurate (checked here at 1e-9; f.stats counts them)
    assert abs(e[-1] - w[idx]) <= 1e-9, (e[-1], w[idx], f.stats)
    o = odmrg.ShiftInvertDMRG(arr, 64, offset=offset, seed=5)
    np.testing.assert_allclose(e[-1], o.run(tol=1e-8, max_sweep=20)[-1], atol=1e-9)
    psi = f.restored_mps.tensors[0].cpu().numpy()
    for a in f.restored_mps.tensors[1:]:
        psi = np.tensordot(psi, a.cpu().numpy(), axes=([-1], [0]))
    psi = psi.reshape(-1)
    # up to a global sign; the reference's 1e-5 perturbation step limits the vector to ~1e-6
    assert min(np.abs(psi - V[:, idx]).max(), np.abs(psi + V[:, idx]).max()) < 5e-6
    r = f.restored_mps
    e_r = expectation_value(r, tg.MatrixProductOperator(base)) / expectation_value(r)
    np.testing.assert_allclose(e_r, e[-1], atol=1e-6)
    assert isinstance(f.variance(), float)
