"""tSDRG tree measurements (tnpy/tsdrg.py:711-1028) against exact diagonalisation, following
the reference's own test class (tests/test_tsdrg.py:166-278): RandomHeisenberg(n=8, h=0.5) with
chi = 2^8 (no truncation, so the tree holds exact eigenstates); tolerance 1e-12 as there."""
import numpy as np
import pytest

from oracle import ed as oed
from oracle import models as om

pytestmark = pytest.mark.gpu

N = 8
SZ = np.diag([0.5, -0.5])


@pytest.fixture(scope="module")
def system(cuda):
    import tnpy_gb300 as tg

    # the reference draws the fields unseeded; a fixed seed stands in for it here
    mpo_arrays = om.random_heisenberg_mpo(N, 0.5, seed=2024)
    mpo = tg.MatrixProductOperator(mpo_arrays)
    t = tg.TSDRG(mpo, chi=2**N)
    t.run()
    ed = oed.ExactDiagonalization(mpo_arrays)
    return t, ed, mpo_arrays


def _psi(ed, level):
    return ed.evecs[:, level]


def _op(op, site):
    return np.kron(np.kron(np.eye(2**site), op), np.eye(2 ** (N - site - 1)))


def test_sandwich(system):
    t, ed, _ = system
    m = t.measurements
    np.testing.assert_allclose(t.evals, np.diag(m.sandwich(t.mpo).cpu().numpy()), atol=1e-12)
    np.testing.assert_allclose(np.identity(t.chi), m.sandwich().cpu().numpy(), atol=1e-12)


def test_expectation_value_and_variance(system):
    t, ed, _ = system
    np.testing.assert_allclose(np.sort(t.measurements.expectation_value(t.mpo)), ed.evals, atol=1e-12)
    # exact eigenstates: zero energy variance on every level
    np.testing.assert_allclose(t.measurements.variance(t.mpo), np.zeros(2**N), atol=1e-10)


@pytest.mark.parametrize("site", list(range(N - 1)))
def test_reduced_density_matrix_and_entropy(system, site):
    t, ed, _ = system
    psi = _psi(ed, 0).reshape(2 ** (site + 1), -1)
    s = np.linalg.svd(psi, compute_uv=False)
    rho_ref = s**2
    rdm = t.measurements.reduced_density_matrix(site=site, level_idx=0)
    w = np.linalg.eigvalsh(rdm)[::-1]
    np.testing.assert_allclose(w[: rho_ref.size], rho_ref[: w.size], atol=1e-12)
    with np.errstate(divide="ignore", invalid="ignore"):
        ent_ref = np.nan_to_num(-rho_ref @ np.log(rho_ref))
    np.testing.assert_allclose(t.measurements.entanglement_entropy(site=site, level_idx=0, nan_to_num=True),
                               ent_ref, atol=1e-10)


@pytest.mark.parametrize("site", list(range(N)))
def test_one_point_function(system, site):
    t, ed, _ = system
    ref = _psi(ed, 0) @ _op(SZ, site) @ _psi(ed, 0)
    np.testing.assert_allclose(t.measurements.one_point_function(SZ, site, level_idx=0), ref, atol=1e-12)


@pytest.mark.parametrize("site1,site2", [(1, 3), (2, 6), (4, 3)])
def test_two_point_functions(system, site1, site2):
    t, ed, _ = system
    psi = _psi(ed, 0)
    two = psi @ _op(SZ, site1) @ _op(SZ, site2) @ psi
    m = t.measurements
    np.testing.assert_allclose(m.two_point_function(SZ, SZ, site1, site2, level_idx=0), two, atol=1e-12)
    conn = two - (psi @ _op(SZ, site1) @ psi) * (psi @ _op(SZ, site2) @ psi)
    np.testing.assert_allclose(m.connected_two_point_function(SZ, SZ, site1, site2, level_idx=0), conn, atol=1e-12)


def test_excited_level_and_errors(system):
    t, ed, _ = system
    m = t.measurements
    # level 5 (exact tree, non-degenerate spectrum with h != 0)
    order = np.argsort(t.evals)
    lvl = int(order[5])
    psi = ed.evecs[:, 5]
    np.testing.assert_allclose(m.one_point_function(SZ, 2, level_idx=lvl), psi @ _op(SZ, 2) @ psi, atol=1e-10)
    with pytest.raises(ValueError):
        m.reduced_density_matrix(site=N - 1, level_idx=0)
    with pytest.raises(ValueError):
        m.one_point_function(SZ, 0, level_idx=2**N)
    with pytest.raises(ValueError):
        m.two_point_function(SZ, SZ, 3, 3, level_idx=0)


def test_measurements_need_a_run(cuda):
    import tnpy_gb300 as tg

    t = tg.TSDRG(tg.model.RandomHeisenberg(6, h=0.5, seed=1).mpo, chi=4)
    with pytest.raises(RuntimeError):
        _ = t.measurements
