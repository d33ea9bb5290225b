"""Exact diagonalisation on the device (tnpy/exact_diagonalization.py:10-250): the dense
Hamiltonian kernel against the reference's exact matrices (tests/test_operators.py:42-88), the
spectrum against its known answers (tests/test_exact_diagonalization.py:10-42, the tSDRG
notebook's n=6 spectrum) and against numpy at n=10 and n=12, and the measurements against
numpy on the same eigenvectors."""
import numpy as np
import pytest

from oracle import models as om
from oracle import operators as oops

pytestmark = pytest.mark.gpu

SZ = np.diag([0.5, -0.5])


def _mpo(tg, spec):
    if spec["model"] == "random_heisenberg":
        arr = om.random_heisenberg_mpo(spec["n"], spec["h"], seed=spec.get("seed"))
    else:
        arr = om.xxz_mpo(spec["n"], spec["delta"])
    return tg.MatrixProductOperator(arr), arr


def test_full_hamiltonian_matches_golden(cuda, golden):
    import tnpy_gb300 as tg
    from tnpy_gb300.exact_diagonalization import full_hamiltonian

    for spec in golden["full_hamiltonian"]:
        mpo, _ = _mpo(tg, spec)
        H = full_hamiltonian(mpo).cpu().numpy()
        np.testing.assert_array_equal(H, np.array(spec["matrix"]))


def test_ed_n2_known_answer(cuda, golden):
    import tnpy_gb300 as tg

    spec = golden["ed_n2"]
    mpo, _ = _mpo(tg, spec)
    ed = tg.ExactDiagonalization(mpo)
    np.testing.assert_allclose(ed.evals, spec["evals"], atol=1e-12)
    v = ed.evecs.cpu().numpy()
    # the singlet is unique up to sign; the triplet only as a subspace
    ref = np.array(spec["evecs"])
    assert abs(abs(v[:, 0] @ ref[:, 0]) - 1) < 1e-12
    np.testing.assert_allclose(v[:, 1:] @ v[:, 1:].T, ref[:, 1:] @ ref[:, 1:].T, atol=1e-12)


def test_ed_notebook_spectrum(cuda, golden):
    import tnpy_gb300 as tg

    spec = golden["notebook_ed"]
    mpo, _ = _mpo(tg, spec)
    ed = tg.ExactDiagonalization(mpo)
    k = len(spec["evals"])
    np.testing.assert_allclose(ed.evals[:k], spec["evals"], atol=1e-8)


@pytest.mark.parametrize("n", [10, 12])
def test_ed_vs_numpy_and_measurements(cuda, n):
    import tnpy_gb300 as tg

    arr = om.random_heisenberg_mpo(n, 0.5, seed=n)
    ed = tg.ExactDiagonalization(tg.MatrixProductOperator(arr))
    H = oops.full_hamiltonian(arr)
    w, V = np.linalg.eigh(H)
    np.testing.assert_allclose(ed.evals, w, atol=1e-11)
    v = ed.evecs.cpu().numpy()
    assert np.abs(v.T @ v - np.eye(2**n)).max() < 1e-11
    assert np.abs(H @ v[:, :8] - v[:, :8] * ed.evals[:8]).max() < 1e-11
    psi = V[:, 0] * np.sign(V[:, 0] @ v[:, 0])
    for site in (0, n // 2 - 1, n - 2):
        shape = (2 ** (site + 1), -1) if site < n // 2 else (-1, 2 ** (n - site - 1))
        rho_ref = np.linalg.svd(psi.reshape(shape), compute_uv=False) ** 2
        np.testing.assert_allclose(ed.reduced_density_matrix(site, 0), rho_ref, atol=1e-12)
        with np.errstate(divide="ignore", invalid="ignore"):
            ent = np.nan_to_num(-rho_ref @ np.log(rho_ref))
        np.testing.assert_allclose(ed.entanglement_entropy(site, 0, nan_to_num=True), ent, atol=1e-10)
    op = lambda o, s: np.kron(np.kron(np.eye(2**s), o), np.eye(2 ** (n - s - 1)))  # noqa: E731
    np.testing.assert_allclose(ed.one_point_function(SZ, 3, 0), psi @ op(SZ, 3) @ psi, atol=1e-12)
    two = psi @ op(SZ, 2) @ op(SZ, 6) @ psi
    np.testing.assert_allclose(ed.two_point_function(SZ, SZ, 6, 2, 0), two, atol=1e-12)
    conn = two - (psi @ op(SZ, 2) @ psi) * (psi @ op(SZ, 6) @ psi)
    np.testing.assert_allclose(ed.connected_two_point_function(SZ, SZ, 2, 6, 0), conn, atol=1e-12)
    np.testing.assert_allclose(ed.variance()[:16], np.zeros(16), atol=1e-10)
    with pytest.raises(ValueError):
        ed.two_point_function(SZ, SZ, 3, 3, 0)
    with pytest.raises(ValueError):
        ed.reduced_density_matrix(n - 1, 0)


def test_ed_size_limit(cuda):
    import tnpy_gb300 as tg

    with pytest.raises(ResourceWarning):
        tg.ExactDiagonalization(tg.model.XXZ(13, 0.5).mpo)
