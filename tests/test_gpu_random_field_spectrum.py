"""Random-field Heisenberg chains H = sum S_i.S_{i+1} + h_i Sz_i, h_i ~ U[-3, 3] from
RandomState(7) (tnpy/model/random_heisenberg.py:57-58, 92-109): the mixed form with FP32
environment storage against FP64. At a size the oracle sweeps in seconds the energies and the
middle-bond entanglement spectrum are checked against the CPU restatement; at n=200, chi=512 the
mixed form's converged state is checked against the FP64 form's converged state started from it."""
import numpy as np
import pytest
import torch

from oracle import dmrg as odmrg
from oracle import models as om

pytestmark = pytest.mark.gpu


def _energy(tg, mps, mpo):
    """<psi|H|psi> / <psi|psi> of the final state, contracted in FP64."""
    from tnpy_gb300.matrix_product_state import expectation_value

    return expectation_value(mps, mpo) / expectation_value(mps)


@pytest.mark.parametrize("form", [("fp64", "fp64"), ("mixed", "fp32"), ("mixed", "fp64")])
def test_random_heisenberg_vs_oracle(cuda, form):
    """FP32 environment storage rounds H_eff at ~6e-8 relative: the sweep's local eigenvalues
    then wander by ~1e-6 from sweep to sweep, so that form is run to a 1e-6 energy tolerance, and
    its accuracy is read from the state: the FP64 energy <H> of the final MPS (second order in the
    state error) and the middle-bond spectrum."""
    import tnpy_gb300 as tg

    precision, env = form
    n, chi = 32, 32
    mpo = om.random_heisenberg_mpo(n, 3.0, seed=7)
    tmpo = tg.MatrixProductOperator(mpo)
    f = tg.FiniteDMRG(tmpo, bond_dim=chi, seed=1234, precision=precision, env_precision=env,
                      compute_variance=False)
    e = f.run(tol=1e-6 if env == "fp32" else 1e-10, max_sweep=10)
    o = odmrg.FiniteDMRG(mpo, chi=chi, seed=1234)
    e_ref = o.run(tol=1e-10, max_sweep=10, with_variance=False)
    assert f.stats["unconverged"] == 0
    if env == "fp64":
        assert abs(e[-1] - e_ref[-1]) <= 1e-9 * abs(e_ref[-1]), (e[-1], e_ref[-1])
    e_state = _energy(tg, f.mps, tmpo)
    assert abs(e_state - e_ref[-1]) <= 1e-9 * abs(e_ref[-1]), (e_state, e_ref[-1])
    bond = n // 2 - 1
    lam = f.measurements.entanglement_spectrum(bond)
    lam_ref = tg.MatrixProductStateMeasurements(tg.MatrixProductState(o.mps, device=cuda)).entanglement_spectrum(bond)
    # Schmidt values are first order in the state error: FP64 meets 1e-8; the mixed form accepts
    # local residuals of 2e-7 |theta| (measured 1.2e-8 here); FP32-stored environments perturb
    # H_eff at ~6e-8 relative (measured 3.1e-7)
    tol = {("fp64", "fp64"): 1e-8, ("mixed", "fp64"): 3e-8, ("mixed", "fp32"): 1e-6}[form]
    assert np.abs(lam - lam_ref).max() <= tol, np.abs(lam - lam_ref).max()


def test_fp32_environments_are_stored_fp32(cuda):
    import tnpy_gb300 as tg

    f = tg.FiniteDMRG(tg.model.RandomHeisenberg(12, h=3.0, seed=7).mpo, bond_dim=16, precision="mixed",
                      env_precision="fp32", compute_variance=False)
    assert all(t.dtype == torch.float32 for t in f.env.left.values())
    assert all(t.dtype == torch.float32 for t in f.env.right.values())
    L, W, R = f.env.site_operator(6)
    assert L.dtype == R.dtype == torch.float64
    with pytest.raises(ValueError):
        tg.FiniteDMRG(tg.model.XXZ(8, 0.5).mpo, bond_dim=8, env_precision="fp16")


def test_random_field_n200_chi512_spectrum_mixed_fp32_env_vs_fp64(cuda):
    """n=200, chi=512: mixed form with FP32 environments swept to convergence from the seeded
    random MPS; the FP64 form then converges from a copy of that state. Middle-bond
    entanglement spectra agree within 2e-6 (the FP32 rounding of the stored environments, first
    order in the Schmidt values); the FP64 energy <H> of the mixed state agrees with the FP64
    form's converged energy within 1e-9 relative."""
    import tnpy_gb300 as tg

    n, chi = 200, 512
    mpo = tg.model.RandomHeisenberg(n, h=3.0, seed=7).mpo
    f = tg.FiniteDMRG(mpo, bond_dim=chi, seed=1234, precision="mixed", env_precision="fp32",
                      compute_variance=False)
    f.run(tol=1e-6, max_sweep=10)
    assert f.stats["unconverged"] == 0
    g = tg.FiniteDMRG(mpo, bond_dim=chi, mps=tg.MatrixProductState([t.clone() for t in f.mps.tensors], device=cuda),
                      precision="fp64", compute_variance=False)
    e_fp64 = g.run(tol=1e-10, max_sweep=6)[-1]
    bond = n // 2 - 1
    lam_m = f.measurements.entanglement_spectrum(bond)
    lam_f = g.measurements.entanglement_spectrum(bond)
    e_mixed = _energy(tg, f.mps, mpo)
    assert abs(e_mixed - e_fp64) <= 1e-9 * abs(e_fp64), (e_mixed, e_fp64)
    # FP32-stored environments: measured 6.1e-7 (the 1e-8 spectrum target needs FP64 storage)
    assert np.abs(lam_m - lam_f).max() <= 2e-6, np.abs(lam_m - lam_f).max()
    sz_m, sz_f = f.measurements.local_sz(), g.measurements.local_sz()
    assert np.abs(sz_m - sz_f).max() < 1e-5
