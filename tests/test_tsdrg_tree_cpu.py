"""Host-side tSDRG structures without a GPU: the isometry tree (TensorTree, tsdrg.py:64-441)
on the 4-site merge sequence of the reference's own tree tests (tests/test_tsdrg.py:15-76):
sites 1+2 -> 4, 0+4 -> 5, 5+3 -> 6; and the truncation gap (tsdrg.py:594-605) against the
oracle's restatement."""
import numpy as np
import pytest

from oracle import tsdrg as otsdrg
from tnpy_gb300.tsdrg import TensorTree, _gap


@pytest.fixture
def tree():
    t = TensorTree(4)
    t.fuse(left_id=1, right_id=2, new_id=4, data=np.zeros((2, 2, 4)))
    t.fuse(left_id=0, right_id=4, new_id=5, data=np.zeros((2, 4, 8)))
    t.fuse(left_id=5, right_id=3, new_id=6, data=np.zeros((8, 2, 16)))
    return t


def test_leaves_nodes_layers(tree):
    assert all(tree[s].is_leaf for s in range(4))
    assert not tree[5].is_leaf and not tree[4].is_leaf
    assert tree.n_nodes == 7 and tree.n_leaves == 4
    assert tree.n_layers == 4
    assert tree.root_id == 6


def test_structure(tree):
    assert tree.root.left is tree[5] and tree.root.right is tree[3]
    assert tree[5].left is tree[0] and tree[5].right is tree[4]
    assert tree[4].left is tree[1] and tree[4].right is tree[2]


def test_horizon_follows_the_merges():
    t = TensorTree(4)
    assert t.horizon == [0, 1, 2, 3]
    t.fuse(1, 2, 4, None)
    assert t.horizon == [0, 4, 3]
    t.fuse(0, 4, 5, None)
    assert t.horizon == [5, 3]
    t.fuse(5, 3, 6, None)
    assert t.horizon == [6]


def test_no_fuse_on_a_grown_tree(tree):
    with pytest.raises(RuntimeError):
        tree.fuse(left_id=6, right_id=5, new_id=7, data=None)


def test_root_needed_before_queries():
    t = TensorTree(3)
    with pytest.raises(KeyError):
        _ = t.root
    with pytest.raises(KeyError):
        t.find_path(0)


def test_find_path(tree):
    assert tree.find_path(0) == [6, 5]
    assert tree.find_path(4) == [6, 5]
    assert tree.find_path(2) == [6, 5, 4]
    assert tree.find_path(2, return_itself=True) == [6, 5, 4, 2]
    for missing in (7, -1):
        with pytest.raises(KeyError):
            tree.find_path(missing)


def test_common_ancestor(tree):
    assert tree.common_ancestor(1, 2) == [6, 5, 4]
    assert tree.common_ancestor(0, 2) == [6, 5]
    assert tree.common_ancestor(0, 4) == [6, 5]
    assert tree.common_ancestor(2, 3) == [6]
    assert tree.common_ancestor(0, 1, lowest=True) == 5
    assert tree.common_ancestor(1, 3, lowest=True) == 6


@pytest.mark.parametrize("size,chi", [(16, 4), (5, 4), (4, 4), (3, 8), (2, 1)])
def test_truncation_gap_matches_oracle(size, chi):
    evals = np.sort(np.random.RandomState(size * 31 + chi).standard_normal(size))
    assert _gap(evals, chi) == otsdrg.truncation_gap(evals, chi)
