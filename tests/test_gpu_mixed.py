"""Split-BF16 tcgen05 path: the tensor-core GEMM, the mixed matvec, and the refined
mixed-precision Davidson / fDMRG against FP64."""
import numpy as np
import pytest
import torch

from oracle import dmrg as odmrg
from oracle import models as om
from oracle import mps as omps

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 260, 200), (1000, 512, 700), (5, 7, 3)])
def test_gemm_bf16x3(cuda, m, n, k):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(m + n + k)
    a, b = rng.standard_normal((m, k)), rng.standard_normal((n, k))
    c = K.gemm_bf16x3(_t(a, cuda), _t(b, cuda)).cpu().numpy()
    ref = a @ b.T
    # three-term split-BF16 products: ~2^-16 relative per product (plain BF16 would be ~2^-8)
    assert np.abs(c - ref).max() <= 2e-4 * np.sqrt(k) * 0.05 + 1e-5 * np.abs(ref).max(), np.abs(c - ref).max()


@pytest.mark.parametrize("chi_l,chi_r", [(16, 16), (64, 64), (128, 96), (256, 256)])
def test_matvec1_mixed(cuda, chi_l, chi_r):
    import tnpy_gb300.kernels as K

    rng = np.random.RandomState(chi_l)
    L = rng.standard_normal((chi_l, 5, chi_l))
    R = rng.standard_normal((chi_r, 5, chi_r))
    W = om.uniform(om.xxz_mpo(6, -0.5))[2]
    x = rng.standard_normal((chi_l, 2, chi_r))
    y = K.matvec1(_t(L, cuda), _t(W, cuda), _t(R, cuda), _t(x, cuda), precision="mixed").cpu().numpy()
    ref = omps.one_site_matvec(L, W, R, x)
    rel = np.abs(y - ref).max() / np.abs(ref).max()
    assert rel < 1e-4, rel


@pytest.mark.parametrize("chi", [32, 64])
def test_davidson_mixed_defect_corrected(cuda, chi):
    import tnpy_gb300.kernels as K

    mpo = om.xxz_mpo(16, -0.5)
    m = omps.random_mps(16, chi, 2, seed=chi)
    env = omps.Environment(mpo, m)
    site = 8
    L, W, R = env.left[site], om.uniform(mpo)[site], env.right[site]
    w = np.linalg.eigvalsh(omps.one_site_full_matrix(L, W, R))
    x64 = _t(m[site], cuda).clone()
    e64, _, its64, _ = K.davidson1(_t(L, cuda), _t(W, cuda), _t(R, cuda), x64, tol=1e-10)
    st64 = K.davidson1_stats()
    assert st64["phase1"] == its64 and st64["anchored"] == 0 and st64["anchors"] == 0, st64
    xm = _t(m[site], cuda).clone()
    em, rn, its, ok = K.davidson1(_t(L, cuda), _t(W, cuda), _t(R, cuda), xm, tol=1e-10, precision="mixed")
    st = K.davidson1_stats()
    assert st["phase1"] + st["anchored"] == its and st["anchors"] >= 1, st
    np.testing.assert_allclose(e64, w[0], rtol=1e-12)
    # the FP64 Rayleigh quotient of the mixed eigenvector: error quadratic in the vector error
    assert abs(em - w[0]) <= 1e-9 * abs(w[0]), (em, w[0], rn)


def test_fdmrg_mixed_matches_fp64(cuda):
    """XXZ(32, -0.5), chi=32: refined mixed precision within |dE|/|E| <= 1e-9 of the FP64 oracle."""
    import tnpy_gb300 as tg

    mpo = om.xxz_mpo(32, -0.5)
    f = tg.FiniteDMRG(tg.MatrixProductOperator(mpo), bond_dim=32, seed=1234, precision="mixed",
                      compute_variance=False)
    e = f.run(tol=1e-10, max_sweep=10)
    o = odmrg.FiniteDMRG(mpo, chi=32, seed=1234)
    e_ref = o.run(tol=1e-10, max_sweep=10, with_variance=False)
    assert abs(e[-1] - e_ref[-1]) <= 1e-9 * abs(e_ref[-1]), (e[-1], e_ref[-1])
    sz = f.measurements.local_sz()
    assert np.max(np.abs(sz - omps.local_sz(o.mps))) < 1e-4


@pytest.mark.parametrize("chi", [128, 256])
def test_davidson_mixed_from_random_start(cuda, chi):
    """Local problem of a swept chain solved from a random start vector (far from its ground
    state): the mixed solver must still converge, to the FP64 solver's eigenvalue."""
    import torch

    import tnpy_gb300 as tg
    from tnpy_gb300 import kernels as K

    f = tg.FiniteDMRG(tg.model.XXZ(24, -0.5).mpo, bond_dim=chi, seed=3, compute_variance=False, precision="mixed")
    f.sweep(tg.Direction.RIGHTWARD, tol=1e-8)
    site = 12
    L, W, R = f.env.site_operator(site)
    shape = f.mps.tensors[site].shape
    g = torch.Generator(device="cpu").manual_seed(9)
    x0 = torch.randn(shape, generator=g, dtype=torch.float64).to(cuda)
    em, rm, itm, okm = K.davidson1(L, W, R, x0.clone(), tol=1e-10, precision="mixed", max_iter=400)
    ef, rf, itf, okf = K.davidson1(L, W, R, x0.clone(), tol=1e-10, precision="fp64", max_iter=400)
    assert okm and okf, (em, rm, itm, ef, rf, itf)
    assert abs(em - ef) <= 1e-9 * abs(ef), (em, ef)


@pytest.fixture(scope="module", params=[512, 1024])
def swept_chain(request, cuda):
    """XXZ(24, -0.5) at chi = 512 / 1024 (the middle bonds reach chi) after one rightward
    mixed-precision sweep from the seeded random MPS: the local operators of a real sweep."""
    import tnpy_gb300 as tg

    chi = request.param
    f = tg.FiniteDMRG(tg.model.XXZ(24, -0.5).mpo, bond_dim=chi, seed=11, compute_variance=False,
                      precision="mixed")
    f.sweep(tg.Direction.RIGHTWARD, tol=1e-8)
    yield chi, f
    del f
    torch.cuda.empty_cache()


@pytest.mark.parametrize("start", ["site_tensor", "random"])
def test_davidson_mixed_hard_start_large_chi(cuda, swept_chain, start):
    """chi = 512 and 1024 local problems from a far-off start: the middle site's tensor after the
    sweep has moved past it (a left-orthonormal gauge tensor, as in a bench chain's middle site)
    and a random vector. The mixed solver must converge, to the FP64 solver's eigenvalue within
    |dE|/|E| <= 1e-9, and report convergence."""
    from tnpy_gb300 import kernels as K

    chi, f = swept_chain
    site = 12
    L, W, R = f.env.site_operator(site)
    assert L.shape[0] == chi and R.shape[0] == chi
    if start == "random":
        g = torch.Generator(device="cpu").manual_seed(chi + 5)
        x0 = torch.randn(f.mps.tensors[site].shape, generator=g, dtype=torch.float64).to(cuda)
    else:
        x0 = f.mps.tensors[site].clone()
    em, rm, itm, okm = K.davidson1(L, W, R, x0.clone(), tol=1e-10, precision="mixed", max_iter=400)
    stm = K.davidson1_stats()
    ef, rf, itf, okf = K.davidson1(L, W, R, x0.clone(), tol=1e-10, precision="fp64", max_iter=400)
    assert okf, (ef, rf, itf)
    assert okm, (em, rm, itm, stm)
    assert abs(em - ef) <= 1e-9 * abs(ef), (em, ef, stm)
