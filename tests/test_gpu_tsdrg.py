"""tSDRG on the GPU against the CPU oracle, the reference's known answers and ED."""
import numpy as np
import pytest
import torch

from oracle import ed as oed
from oracle import models as om
from oracle import tsdrg as ots

pytestmark = pytest.mark.gpu


def test_block_hamiltonian_kat(cuda, golden):
    """tests/test_tsdrg.py:116-128 of the reference (n=8, h=0, every bond)."""
    import tnpy_gb300 as tg
    from tnpy_gb300.tsdrg import block_hamiltonians

    g = golden["tsdrg_block"]
    w = tg.model.RandomHeisenberg(g["n"], g["h"]).mpo.device_tensors(cuda)
    mats, _ = block_hamiltonians([(w[s], w[s + 1]) for s in range(5)], cuda)
    for m in mats:
        np.testing.assert_array_equal(m.cpu().numpy(), np.array(g["block_hamiltonian"]))


def test_projector_matches_oracle(cuda):
    from tnpy_gb300.tsdrg import project

    rng = np.random.RandomState(0)
    for dl, dr, m1, m2, k in [(1, 5, 2, 2, 4), (5, 5, 8, 2, 16), (5, 1, 32, 32, 32), (5, 5, 16, 16, 40)]:
        w1 = rng.standard_normal((dl, 5, m1, m1))
        w2 = rng.standard_normal((5, dr, m2, m2))
        v = np.linalg.qr(rng.standard_normal((m1 * m2, k)))[0]
        (out,) = project([(torch.from_numpy(w1).to(cuda), torch.from_numpy(w2).to(cuda),
                           torch.from_numpy(np.ascontiguousarray(v)).to(cuda))], cuda)
        ref, _ = ots.spectrum_projector(w1, w2, v)
        np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-12 * np.abs(ref).max())


def test_notebook_kat(cuda, golden):
    """docs/source/notebooks/tsdrg.ipynb: RandomHeisenberg(6, 3.0, seed=2021), chi=4."""
    import tnpy_gb300 as tg

    g = golden["notebook_tsdrg"]
    t = tg.TSDRG(tg.model.RandomHeisenberg(g["n"], g["h"], seed=g["seed"]).mpo, chi=g["chi"])
    t.run()
    np.testing.assert_allclose(np.sort(t.evals), g["evals"], atol=1.5e-8)
    merges = [[n.left.node_id, n.right.node_id] for n in t.tree if not n.is_leaf]
    old_to_new = {k: k - 1 if k >= g["n"] else k for k in range(3 * g["n"])}
    assert merges == [[old_to_new[a], old_to_new[b]] for a, b in g["merged_pairs_old_ids"]]
    assert t.tree.root_id == 2 * g["n"] - 2
    with pytest.raises(RuntimeError):
        t.tree.fuse(left_id=t.tree.root_id, right_id=0, new_id=99, data=None)


@pytest.mark.parametrize("n,h,seed", [(4, 0.1, 0), (6, 1.0, 3), (8, 0.5, 11)])
def test_exact_tree_vs_ed(cuda, n, h, seed):
    import tnpy_gb300 as tg

    mpo = tg.model.RandomHeisenberg(n, h, seed=seed).mpo
    t = tg.TSDRG(mpo, chi=2**n)
    t.run()
    np.testing.assert_allclose(np.sort(t.evals), oed.ExactDiagonalization(list(mpo)).evals, atol=1e-10)
    assert t.tree.n_layers >= 2


def _oracle_chain(n, seed, h):
    fields = np.random.RandomState(seed + 1).uniform(-h, h, size=n) if h > 0 else None
    return om.random_coupling_heisenberg_mpo(n, om.random_couplings(n, 1.0, seed), fields=fields)


# Random fields (h > 0) break the SU(2) symmetry of the h = 0 chain: with exact multiplets
# cut by the truncation the kept subspace is not unique and depends on the eigensolver's basis
# inside the multiplet, so parity is checked on non-degenerate chains.
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,chi,seed", [(16, 8, 10000), (24, 4, 10001)])
def test_random_coupling_chain_vs_oracle(cuda, n, chi, seed, precision):
    """Random-coupling Heisenberg chain: same merge order and kept spectrum as the CPU restatement,
    in both precision modes (chi <= 8: every block is a dense solve)."""
    import tnpy_gb300 as tg

    model = tg.model.RandomCouplingHeisenberg(n, delta=1.0, h=0.5, seed=seed)
    t = tg.TSDRG(model.mpo, chi=chi, precision=precision)
    t.run()
    o = ots.TreeTensorNetworkSDRG(_oracle_chain(n, seed, 0.5), chi).run()
    np.testing.assert_allclose(t.evals, o.evals, atol=1e-10)
    assert [[n_.left.node_id, n_.right.node_id, n_.node_id] for n_ in t.tree if not n_.is_leaf] == \
        [list(m) for m in o.merges]


def test_batched_matches_single(cuda):
    import tnpy_gb300 as tg

    seeds = [10000 + r for r in range(5)]
    mpos = [tg.model.RandomCouplingHeisenberg(12, delta=1.0, h=0.5, seed=s).mpo for s in seeds]
    b = tg.BatchedTSDRG(mpos, chi=8).run()
    for s, ev, mg in zip(seeds, b.evals, b.merges):
        o = ots.TreeTensorNetworkSDRG(_oracle_chain(12, s, 0.5), 8).run()
        np.testing.assert_allclose(ev, o.evals, atol=1e-10)
        assert [list(m) for m in mg] == [list(m) for m in o.merges]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("m1,m2,dl,dr,chi", [(32, 32, 5, 5, 32), (32, 2, 5, 1, 32), (16, 16, 1, 5, 16), (8, 16, 5, 5, 8)])
def test_kronecker_eigensolver(cuda, precision, m1, m2, dl, dr, chi):
    """Kronecker-sum subspace eigensolver vs numpy eigh of the dense block Hamiltonian."""
    from tnpy_gb300.tsdrg import kron_eigh

    rng = np.random.RandomState(m1 * 100 + m2)
    w1 = rng.standard_normal((dl, 5, m1, m1))
    w1 = 0.5 * (w1 + w1.transpose(0, 1, 3, 2))
    w2 = rng.standard_normal((5, dr, m2, m2))
    w2 = 0.5 * (w2 + w2.transpose(0, 1, 3, 2))
    h = ots.block_hamiltonian(w1, w2)
    w, v = np.linalg.eigh(h)
    t1, t2 = torch.from_numpy(w1).to(cuda), torch.from_numpy(w2).to(cuda)
    ev, vec, ks, iters = kron_eigh([(t1, t2)], chi, cuda, precision=precision)
    assert int(iters[0]) > 0, "subspace iteration reported no convergence"
    k = ks[0]
    ev, vec = ev.cpu().numpy()[0, :k], vec.cpu().numpy()[0, : m1 * m2, :k]
    np.testing.assert_allclose(ev, w[:k], atol=1e-10 * max(1.0, np.abs(w).max()))
    np.testing.assert_allclose(vec.T @ vec, np.eye(k), atol=1e-12)
    # Ritz vectors carry the subspace error of the filtered iteration; Ritz values are second
    # order in it, hence the 1e-10 above
    assert np.abs(h @ vec - vec * ev).max() < 1e-4 * np.abs(w).max()


def test_chain_kronecker_path_vs_oracle(cuda):
    """chi = 16 chain: blocks up to 256 states go through the Kronecker eigensolver."""
    import tnpy_gb300 as tg

    n, chi, seed = 20, 16, 10002
    t = tg.TSDRG(tg.model.RandomCouplingHeisenberg(n, delta=1.0, h=0.5, seed=seed).mpo, chi=chi)
    t.run()
    o = ots.TreeTensorNetworkSDRG(_oracle_chain(n, seed, 0.5), chi).run()
    np.testing.assert_allclose(t.evals, o.evals, atol=1e-10)
    assert [[n_.left.node_id, n_.right.node_id, n_.node_id] for n_ in t.tree if not n_.is_leaf] == \
        [list(m) for m in o.merges]


def test_chain_n64_chi32_fp64_vs_oracle(cuda):
    """chi = 32 on 64 sites: blocks of up to 1024 states with clustered spectra, solved by the
    two-stage (FP32 then FP64) Kronecker subspace iteration; same merges and energies as the
    numpy eigh restatement."""
    import tnpy_gb300 as tg

    n, chi, seed = 64, 32, 10001
    t = tg.TSDRG(tg.model.RandomCouplingHeisenberg(n, delta=1.0, h=0.5, seed=seed).mpo, chi=chi)
    t.run()
    o = ots.TreeTensorNetworkSDRG(_oracle_chain(n, seed, 0.5), chi).run()
    np.testing.assert_allclose(t.evals, o.evals, atol=1e-9 * np.abs(o.evals).max())
    assert [[n_.left.node_id, n_.right.node_id, n_.node_id] for n_ in t.tree if not n_.is_leaf] == \
        [list(m) for m in o.merges]


@pytest.mark.parametrize("seed", [10000, 10007])
def test_batched_n128_chi32_kept_spectra_vs_one_at_a_time_fp64(cuda, seed):
    """The batched-vs-one-at-a-time comparison of n = 128, chi = 32 chains on the h != 0 variant
    (h = 0 is SU(2) symmetric and chi = 32 cuts
    through exact multiplets, where the kept subspace is not unique): n = 128, chi = 32, delta = 1
    random couplings with fields h_i ~ U[-0.5, 0.5). The batched FP64 run (two realisations in one
    lockstep launch sequence) keeps the same spectra as the one-block-at-a-time FP64 numpy eigh
    restatement within 1e-10, with the same merge order."""
    import tnpy_gb300 as tg

    n, chi = 128, 32
    mpos = [tg.model.RandomCouplingHeisenberg(n, delta=1.0, h=0.5, seed=s).mpo for s in (seed, seed + 1)]
    b = tg.BatchedTSDRG(mpos, chi=chi).run()
    o = ots.TreeTensorNetworkSDRG(_oracle_chain(n, seed, 0.5), chi).run()
    np.testing.assert_allclose(b.evals[0], o.evals, atol=1e-10)
    assert [list(m) for m in b.merges[0]] == [list(m) for m in o.merges]


@pytest.mark.parametrize("variant", ["high_energy", "shift_invert"])
def test_tsdrg_variants_vs_oracle(cuda, variant):
    """HighEnergyTreeTensorNetworkSDRG (tnpy/tsdrg.py:1031-1067) and
    ShiftInvertTreeTensorNetworkSDRG (:1070-1089) against their restatements: kept spectra of
    the last block and the merge order."""
    import tnpy_gb300 as tg

    n, chi = 10, 8
    arr = om.random_heisenberg_mpo(n, 0.5, seed=4)
    mpo = tg.MatrixProductOperator(arr)
    if variant == "high_energy":
        t = tg.HighEnergyTreeTensorNetworkSDRG(mpo, chi=chi)
        o = ots.HighEnergyTreeTensorNetworkSDRG(arr, chi)
    else:
        t = tg.ShiftInvertTreeTensorNetworkSDRG(mpo, chi=chi, offset=0.0)
        o = ots.ShiftInvertTreeTensorNetworkSDRG(arr, chi, 0.0)
    t.run()
    o.run()
    np.testing.assert_allclose(t.evals, o.evals, atol=1e-10)
    assert [[n_.left.node_id, n_.right.node_id, n_.node_id] for n_ in t.tree if not n_.is_leaf] == \
        [list(m) for m in o.merges]
    if variant == "high_energy":
        # the kept states are the highest of the chain: <H> of the root states through the tree
        ev = np.sort(t.measurements.expectation_value(mpo))
        np.testing.assert_allclose(ev, np.sort(o.evals), atol=1e-10)
