"""Pin the CPU oracle against the reference's own known-answer tests (no GPU)."""
import numpy as np
import pytest

from oracle import dmrg, ed, models, mps, operators, tsdrg


def _mpo(entry):
    if entry["model"] == "xxz":
        return models.xxz_mpo(entry["n"], entry["delta"])
    return models.random_heisenberg_mpo(entry["n"], entry["h"], seed=entry.get("seed"))


def test_spin_operators():
    sp, sm, sz, i2, o2 = models.spin_operators()
    np.testing.assert_array_equal(sp + sm, [[0, 1], [1, 0]])
    np.testing.assert_array_equal(-1j * (sp - sm), [[0, -1j], [1j, 0]])


def test_full_hamiltonian_kat(golden):
    for entry in golden["full_hamiltonian"]:
        h = operators.full_hamiltonian(_mpo(entry))
        np.testing.assert_array_equal(h, np.array(entry["matrix"]), err_msg=entry["ref"])


def test_ed_n2_kat(golden):
    g = golden["ed_n2"]
    e = ed.ExactDiagonalization(_mpo(g))
    np.testing.assert_array_equal(e.matrix, np.array(g["matrix"]))
    np.testing.assert_array_equal(e.evals, np.array(g["evals"]))
    # eigenvectors: the degenerate triplet is basis dependent, compare the projector on it
    ref = np.array(g["evecs"])
    np.testing.assert_allclose(np.abs(e.evecs[:, 0]), np.abs(ref[:, 0]), atol=1e-15)
    np.testing.assert_allclose(e.evecs[:, 1:] @ e.evecs[:, 1:].T, ref[:, 1:] @ ref[:, 1:].T, atol=1e-14)


def test_notebook_ed_spectrum(golden):
    g = golden["notebook_ed"]
    e = ed.ExactDiagonalization(_mpo(g))
    np.testing.assert_allclose(e.evals, np.array(g["evals"]), atol=1.5 * 10 ** -g["printed_decimals"])


@pytest.mark.parametrize("h", [0.0, 0.5])
def test_mpo_square(h):
    mpo = models.random_heisenberg_mpo(4, h, seed=3)
    sq = operators.mpo_square(mpo)
    assert sq[0].shape == (25, 2, 2) and sq[1].shape == (25, 25, 2, 2) and sq[3].shape == (25, 2, 2)
    ham = operators.full_hamiltonian(mpo)
    np.testing.assert_allclose(ham @ ham, operators.full_hamiltonian(sq), atol=1e-12)


@pytest.mark.parametrize("site", range(5))
def test_tsdrg_block_hamiltonian_kat(golden, site):
    g = golden["tsdrg_block"]
    w = models.uniform(models.random_heisenberg_mpo(g["n"], g["h"]))
    np.testing.assert_array_equal(tsdrg.block_hamiltonian(w[site], w[site + 1]),
                                  np.array(g["block_hamiltonian"]))


def test_tsdrg_projector_kat(golden):
    g = golden["tsdrg_block"]
    w = models.uniform(models.random_heisenberg_mpo(g["n"], g["h"]))
    evecs = np.array(g["evecs"])
    _, v = tsdrg.spectrum_projector(w[3], w[4], evecs)
    np.testing.assert_array_equal(v, evecs.reshape(2, 2, 4))


def test_tsdrg_notebook_kat(golden):
    """docs/source/notebooks/tsdrg.ipynb: RandomHeisenberg(6, 3.0, seed=2021), chi=4."""
    g = golden["notebook_tsdrg"]
    mpo = models.random_heisenberg_mpo(g["n"], g["h"], seed=g["seed"])
    t = tsdrg.TreeTensorNetworkSDRG(mpo, chi=g["chi"]).run()
    np.testing.assert_allclose(np.sort(t.evals), g["evals"], atol=1.5 * 10 ** -g["printed_decimals"])
    # the notebook numbered new nodes n+step; this code (tsdrg.py:686) uses n+step-1
    old_to_new = {k: k - 1 if k >= g["n"] else k for k in range(3 * g["n"])}
    pairs = [[old_to_new[a], old_to_new[b]] for a, b in g["merged_pairs_old_ids"]]
    assert [[a, b] for a, b, _ in t.merges] == pairs


@pytest.mark.parametrize("n,h,seed", [(4, 0.1, 0), (6, 1.0, 3), (8, 0.5, 11)])
def test_tsdrg_exact_tree_vs_ed(n, h, seed):
    """With chi = 2^n nothing is truncated, so the root spectrum is the ED spectrum."""
    mpo = models.random_heisenberg_mpo(n, h, seed=seed)
    t = tsdrg.TreeTensorNetworkSDRG(mpo, chi=2**n).run()
    np.testing.assert_allclose(np.sort(t.evals), ed.ExactDiagonalization(mpo).evals, atol=1e-12)


def test_fdmrg_vs_ed(golden):
    g = golden["fdmrg_vs_ed"]
    mpo = models.xxz_mpo(g["n"], g["delta"])
    e = ed.ExactDiagonalization(mpo)
    f = dmrg.FiniteDMRG(mpo, chi=g["bond_dim"], seed=7)
    energies = f.run(tol=1e-8, max_sweep=20, with_variance=True)
    np.testing.assert_allclose(energies[-1], e.evals[0], atol=g["atol"])
    # the reference's variance is taken on the unnormalised MPS left by the 1e-5
    # perturbation (finite_dmrg.py:139-141, matrix_product_state.py:367-370); the
    # normalised variance of the converged state is ~0
    nrm = mps.norm_sq(f.mps)
    e_n = mps.expectation(f.mps, mpo) / nrm
    var_n = mps.expectation(f.mps, operators.mpo_square(mpo)) / nrm - e_n**2
    assert abs(var_n) < 1e-7


def test_xxz_sign_convention():
    """Reference XXZ(n, delta=-0.5) is the antiferromagnetic SxSx+SySy+0.5SzSz chain."""
    n = 10
    sp, sm, sz, i2, _ = models.spin_operators()
    sx, sy = (sp + sm) / 2, (sp - sm) / 2j
    h = np.zeros((2**n, 2**n), dtype=complex)
    for i in range(n - 1):
        for a, b, c in ((sx, sx, 1.0), (sy, sy, 1.0), (sz, sz, 0.5)):
            ops = [i2] * n
            ops[i], ops[i + 1] = a, b
            t = ops[0]
            for o in ops[1:]:
                t = np.kron(t, o)
            h += c * t
    e_ref = np.linalg.eigvalsh(operators.full_hamiltonian(models.xxz_mpo(n, -0.5)))
    np.testing.assert_allclose(np.linalg.eigvalsh(h), e_ref, atol=1e-12)
    np.testing.assert_allclose(e_ref[0], -3.590250702986, atol=1e-11)


@pytest.mark.parametrize("n", [6, 8])
@pytest.mark.parametrize("chi", [2, 4, 6])
def test_bond_dims(n, chi):
    """tests/test_matrix_product_state.py:11-37 of the reference."""
    d = 2
    m = mps.random_mps(n, chi, d)
    if n % 2 == 0:
        ref = [min(d**i, chi) for i in range(1, n // 2)]
        ref += [int(min(d ** (n / 2), chi))] + ref[::-1]
    else:
        ref = [min(d**i, chi) for i in range(1, (n + 1) // 2)]
        ref += ref[::-1]
    assert [a.shape[2] for a in m[:-1]] == ref


@pytest.mark.parametrize("site", [2, 3, 4, 6])
def test_split_tensor_invariance(site):
    m = mps.random_mps(8, 10, 2, seed=5)
    two = np.tensordot(m[site], m[site + 1], axes=([2], [0]))
    mps.split_tensor(m, site, rightward=True)
    np.testing.assert_allclose(two, np.tensordot(m[site], m[site + 1], axes=([2], [0])), atol=1e-12)


def test_matvec_matches_full_matrix():
    mpo = models.random_heisenberg_mpo(6, 1.0, seed=4)
    m = mps.random_mps(6, 8, 2, seed=1)
    env = mps.Environment(mpo, m)
    for site in range(6):
        x = np.random.RandomState(site).standard_normal(m[site].shape)
        y = env.matvec(site, x)
        h = env.full_matrix(site)
        np.testing.assert_allclose(y.reshape(-1), h.T @ x.reshape(-1), atol=1e-12)
        np.testing.assert_allclose(h, h.T, atol=1e-12)
        np.testing.assert_allclose(np.diag(h), mps.one_site_diagonal(env.left[site], env.w[site],
                                                                     env.right[site]).reshape(-1),
                                   atol=1e-12)


def test_effective_hamiltonian_projects_full_h():
    """x^T H_eff x equals <Psi|H|Psi> for the MPS with x at the orthogonality centre."""
    n = 8
    mpo = models.xxz_mpo(n, -0.5)
    m = mps.random_mps(n, 16, 2, seed=9)
    env = mps.Environment(mpo, m)
    x = m[0]
    e_eff = float(np.vdot(x, env.matvec(0, x)))
    psi = m[0]
    for a in m[1:]:
        psi = np.tensordot(psi, a, axes=([-1], [0]))
    psi = psi.reshape(-1)
    h = operators.full_hamiltonian(mpo)
    np.testing.assert_allclose(e_eff, psi @ h @ psi, atol=1e-12)
    np.testing.assert_allclose(mps.expectation(m, mpo), psi @ h @ psi, atol=1e-12)
