"""fDMRG on the GPU against the CPU oracle and exact diagonalisation."""
import numpy as np
import pytest

from oracle import dmrg as odmrg
from oracle import ed as oed
from oracle import models as om
from oracle import mps as omps

pytestmark = pytest.mark.gpu


def test_reference_fdmrg_case(cuda, golden):
    """tests/test_finite_dmrg.py:9-23 of the reference: XXZ(10, 0.5), bond_dim=32, vs ED at 1e-8."""
    import tnpy_gb300 as tg

    g = golden["fdmrg_vs_ed"]
    model = tg.model.XXZ(n=g["n"], delta=g["delta"])
    ed = oed.ExactDiagonalization(list(model.mpo))
    fdmrg = tg.FiniteDMRG(model.mpo, bond_dim=g["bond_dim"])
    np.testing.assert_allclose(ed.evals[0], fdmrg.run(tol=1e-8)[-1], atol=g["atol"])


def test_readme_spelling(cuda):
    import tnpy_gb300 as tg

    f = tg.FiniteDMRG(mpo=tg.model.XXZ(8, -0.5).mpo, chi=16)
    e = f.update(tol=1e-8)
    ed = oed.ExactDiagonalization(om.xxz_mpo(8, -0.5))
    np.testing.assert_allclose(e[-1], ed.evals[0], atol=1e-8)
    with pytest.raises(RuntimeError):
        tg.FiniteDMRG(mpo=tg.model.XXZ(8, -0.5).mpo, chi=4).measurements


@pytest.mark.parametrize("n,chi,seed", [(12, 32, 11), (32, 32, 1234)])
def test_fdmrg_matches_oracle(cuda, n, chi, seed):
    """Same seeded MPO and initial MPS: per-sweep energies agree with the CPU restatement;
    n=12 also against ED; n=32 chi=32 is the CPU-runnable configuration."""
    import tnpy_gb300 as tg

    mpo = om.xxz_mpo(n, -0.5)
    f = tg.FiniteDMRG(tg.MatrixProductOperator(mpo), bond_dim=chi, seed=seed, compute_variance=False)
    e_gpu = f.run(tol=1e-10, max_sweep=10)
    o = odmrg.FiniteDMRG(mpo, chi=chi, seed=seed)
    e_cpu = o.run(tol=1e-10, max_sweep=10, with_variance=False)
    assert abs(e_gpu[-1] - e_cpu[-1]) <= 1e-9 * abs(e_cpu[-1]), (e_gpu, e_cpu)
    if n <= 12:
        ed = oed.ExactDiagonalization(mpo)
        np.testing.assert_allclose(e_gpu[-1], ed.evals[0], atol=1e-8)
    sz = f.measurements.local_sz()
    sz_ref = omps.local_sz(o.mps)
    assert np.max(np.abs(sz - sz_ref)) < 1e-6


def test_random_heisenberg_variance(cuda):
    import tnpy_gb300 as tg

    mpo = om.random_heisenberg_mpo(10, 1.0, seed=100)
    f = tg.FiniteDMRG(tg.MatrixProductOperator(mpo), bond_dim=32, seed=3)
    e = f.run(tol=1e-9, max_sweep=12)
    ed = oed.ExactDiagonalization(mpo)
    np.testing.assert_allclose(e[-1], ed.evals[0], atol=1e-8)
    o = odmrg.FiniteDMRG(mpo, chi=32, seed=3)
    o.run(tol=1e-9, max_sweep=12)
    # the reference's variance is on the unnormalised MPS; both paths carry the same bias
    np.testing.assert_allclose(f._variances[-1], o.variances[-1], atol=1e-6)


def test_bond_dimension_ramp(cuda):
    """Enlarging the bonds leaves the state unchanged; sweeps at the larger chi lower the energy
    towards the chi=64 oracle result."""
    import tnpy_gb300 as tg
    from tnpy_gb300.matrix_product_state import expectation_value

    mpo = om.xxz_mpo(20, -0.5)
    tmpo = tg.MatrixProductOperator(mpo)
    f = tg.FiniteDMRG(tmpo, bond_dim=8, seed=2, compute_variance=False)
    for k in range(4):
        f.sweep(tg.Direction.RIGHTWARD if k % 2 == 0 else tg.Direction.LEFTWARD, tol=1e-10)
    e_before = expectation_value(f.mps, tmpo) / expectation_value(f.mps)
    f.enlarge_bond_dim(32)
    assert max(f.mps.bond_dims()) == 32
    e_after = expectation_value(f.mps, tmpo) / expectation_value(f.mps)
    np.testing.assert_allclose(e_after, e_before, atol=1e-10)
    energies = [f.sweep(tg.Direction.RIGHTWARD if k % 2 == 0 else tg.Direction.LEFTWARD, tol=1e-10) for k in range(8)]
    o = odmrg.FiniteDMRG(mpo, chi=32, seed=2)
    e_ref = o.run(tol=1e-10, max_sweep=12, with_variance=False)[-1]
    assert energies[-1] < e_before - 1e-6
    assert abs(energies[-1] - e_ref) <= 1e-7 * abs(e_ref), (energies[-1], e_ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_chi_ramp_with_truncation_error_vs_oracle(cuda, precision):
    """FiniteDMRG.ramp on XXZ(16, -0.5), chi 4 -> 8 -> 16 (two sweeps per stage, then to
    convergence): the final energy and middle-bond Schmidt values match the oracle's fixed-chi
    (16) ground state, and the reported truncation error of the last stage (weight beyond
    chi = 8) is the oracle state's sum_{j > 8} lambda_j^2."""
    import tnpy_gb300 as tg

    n = 16
    mpo = om.xxz_mpo(n, -0.5)
    f = tg.FiniteDMRG(tg.MatrixProductOperator(mpo), bond_dim=4, seed=5, precision=precision, compute_variance=False)
    stages = f.ramp([4, 8, 16], sweeps_per_stage=2, tol=1e-11, max_sweep=20)
    assert [s["chi"] for s in stages] == [4, 8, 16]
    assert [s["sweeps"] for s in stages][:2] == [2, 2]
    assert stages[0]["energy"] > stages[1]["energy"] > stages[2]["energy"] - 1e-12
    assert max(f.mps.bond_dims()) == 16 and f.stats["unconverged"] == 0
    o = odmrg.FiniteDMRG(mpo, chi=16, seed=5)
    e_ref = o.run(tol=1e-11, max_sweep=20, with_variance=False)[-1]
    assert abs(stages[-1]["energy"] - e_ref) <= 1e-9 * abs(e_ref), (stages[-1]["energy"], e_ref)
    bond = n // 2 - 1
    psi = o.mps[0]
    for a in o.mps[1:]:
        psi = np.tensordot(psi, a, axes=([-1], [0]))
    psi = psi.reshape(-1) / np.linalg.norm(psi)
    lam_ref = np.linalg.svd(psi.reshape(2 ** (bond + 1), -1), compute_uv=False)[:16]
    np.testing.assert_allclose(stages[-1]["spectrum"], lam_ref, atol=1e-7)
    tr_ref = float(np.sum(lam_ref[8:] ** 2))
    assert abs(stages[-1]["truncation_error_prev_chi"] - tr_ref) <= 1e-9 + 1e-5 * tr_ref
    assert stages[1]["truncation_error_prev_chi"] > 0.0 and "truncation_error_prev_chi" not in stages[0]
