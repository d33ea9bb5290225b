"""Independent chains swept concurrently (BatchedFiniteDMRG): every chain equals its own
FiniteDMRG run, and against exact diagonalisation for small chains."""
import numpy as np
import pytest

from oracle import ed as oed
from oracle import models as om

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_chains_equal_single_runs(cuda, precision):
    import tnpy_gb300 as tg

    seeds = [100, 101, 102, 103, 104]
    mpos = [tg.model.RandomHeisenberg(16, h=1.0, seed=s).mpo for s in seeds]
    b = tg.BatchedFiniteDMRG(mpos, bond_dim=16, workers=3, seed=7, compute_variance=False, precision=precision)
    energies = b.run(tol=1e-10, max_sweep=6)
    assert len(energies) == len(seeds)
    for c, mpo in enumerate(mpos):
        f = tg.FiniteDMRG(mpo, 16, seed=7, compute_variance=False, precision=precision)
        ref = f.run(tol=1e-10, max_sweep=6)
        # same kernels, fixed reduction orders: the stream a chain runs on does not change its arithmetic
        assert energies[c] == pytest.approx(ref, abs=1e-12, rel=0), (c, energies[c], ref)


def test_batched_chains_vs_ed(cuda):
    import tnpy_gb300 as tg

    seeds = [100, 101, 102]
    mpos = [om.random_heisenberg_mpo(10, 1.0, seed=s) for s in seeds]
    b = tg.BatchedFiniteDMRG([tg.MatrixProductOperator(m) for m in mpos], chi=32, workers=2, compute_variance=False)
    energies = b.run(tol=1e-10, max_sweep=10)
    for m, e in zip(mpos, energies):
        np.testing.assert_allclose(e[-1], oed.ExactDiagonalization(m).evals[0], atol=1e-8)
    assert all(1 <= s <= 10 for s in b.sweeps)


def test_batched_needs_chains():
    import tnpy_gb300 as tg

    with pytest.raises(ValueError):
        tg.BatchedFiniteDMRG([], bond_dim=8)
