"""Host-side checks that need no GPU: the C ABI library loads and exports every symbol of
include/tnx.h, argument validation returns status codes, and the host-side model / MPO
mirror matches the oracle."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _header_functions():
    text = (ROOT / "include" / "tnx.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tnx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    so = ROOT / "tnpy_gb300" / "libtnx.so"
    if not so.exists():
        import __graft_entry__

        __graft_entry__.build()
    return ctypes.CDLL(str(so))


def test_header_symbols_exported(lib):
    names = _header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    lib.tnx_status_string.restype = ctypes.c_char_p
    assert lib.tnx_status_string(0) == b"ok"
    assert lib.tnx_status_string(3) == b"workspace too small"


def test_workspace_queries_are_host_only(lib):
    f = lib.tnx_matvec1_workspace_bytes
    f.restype = ctypes.c_size_t
    f.argtypes = [ctypes.c_int64] * 5 + [ctypes.c_int]
    n = f(1024, 2, 1024, 5, 5, 0)
    assert n >= 2 * 5 * 1024 * 2 * 1024 * 8
    g = lib.tnx_davidson1_workspace_bytes
    g.restype = ctypes.c_size_t
    g.argtypes = [ctypes.c_int64] * 5 + [ctypes.c_int, ctypes.c_int]
    assert g(64, 2, 64, 5, 5, 24, 0) > 2 * 24 * 64 * 2 * 64 * 8


def test_davidson_stats_host_only(lib):
    """The solver statistics are host-side, per thread: readable without a GPU."""
    import tnpy_gb300._lib as L

    out = (ctypes.c_int * 4)()
    assert L.lib.tnx_davidson1_stats(out) == L.TNX_OK
    assert all(v >= 0 for v in out)
    assert L.lib.tnx_davidson1_stats(None) == L.TNX_ERR_INVALID_ARG


def test_null_pointers_rejected_without_gpu(lib):
    import tnpy_gb300._lib as L

    st = L.lib.tnx_matvec1(None, None, None, None, None, 4, 2, 4, 5, 5, 0, None, 0, None)
    assert st == L.TNX_ERR_INVALID_ARG
    assert b"null" in L.lib.tnx_last_error()
    st = L.lib.tnx_env_update(2, None, None, None, None, 4, 2, 4, 5, 5, 0, None, 0, None)
    assert st == L.TNX_ERR_INVALID_ARG
    st = L.lib.tnx_qr(None, 4, 8, None, None, None, 0, None)
    assert st == L.TNX_ERR_INVALID_ARG


def test_error_mapping():
    import tnpy_gb300._lib as L

    with pytest.raises(ValueError):
        L.check("x", L.TNX_ERR_SHAPE)
    with pytest.raises(NotImplementedError):
        L.check("x", L.TNX_ERR_UNSUPPORTED)
    with pytest.raises(L.NotConverged):
        L.check("x", L.TNX_ERR_NOT_CONVERGED)


@pytest.mark.parametrize("n", [2, 3, 7])
def test_models_match_oracle(n):
    import tnpy_gb300 as tg
    from oracle import models as om

    for a, b in zip(tg.model.XXZ(n, 0.5).mpo, om.xxz_mpo(n, 0.5)):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(tg.model.RandomHeisenberg(n, 1.5, seed=4).mpo, om.random_heisenberg_mpo(n, 1.5, seed=4)):
        np.testing.assert_array_equal(a, b)
    rc = tg.model.RandomCouplingHeisenberg(n, delta=1.0, seed=10007)
    for a, b in zip(rc.mpo, om.random_coupling_heisenberg_mpo(n, om.random_couplings(n, 1.0, 10007))):
        np.testing.assert_array_equal(a, b)


def test_full_hamiltonian_and_square_match_oracle(golden):
    import tnpy_gb300 as tg
    from oracle import operators as oo

    for entry in golden["full_hamiltonian"]:
        mpo = (tg.model.XXZ(entry["n"], entry["delta"]) if entry["model"] == "xxz"
               else tg.model.RandomHeisenberg(entry["n"], entry["h"])).mpo
        np.testing.assert_array_equal(tg.FullHamiltonian(mpo).matrix, np.array(entry["matrix"]))
    mpo = tg.model.RandomHeisenberg(4, 0.5, seed=1).mpo
    sq = mpo.square()
    assert sq[0].shape == (25, 2, 2) and sq[1].shape == (25, 25, 2, 2)
    h = tg.FullHamiltonian(mpo).matrix
    np.testing.assert_allclose(h @ h, tg.FullHamiltonian(sq).matrix, atol=1e-12)
    np.testing.assert_array_equal(-1 * tg.FullHamiltonian(mpo).matrix, tg.FullHamiltonian(-1 * mpo).matrix)
    for a, b in zip(sq, oo.mpo_square(list(mpo))):
        np.testing.assert_allclose(a, b, atol=0)


def test_product_requires_cuda_for_state():
    import torch

    import tnpy_gb300 as tg

    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    with pytest.raises(RuntimeError):
        tg.MatrixProductState.random(4, 2, 2)


def test_mps_npz_round_trip_and_reference_layout(tmp_path):
    """MatrixProductState.save / load in .npz (tnpy/matrix_product_state.py:118-168): keys are
    the site tags I0..I{n-1}, tensors in 'lpr' order with the boundary sites 2-index ((d, chi)
    and (chi, d)); a file whose keys are in site order, as the reference writes and reads it
    (:130, :158), loads site by site, and so do more than ten sites (I10 after I9)."""
    import numpy as np
    import pytest

    import tnpy_gb300 as tg

    rng = np.random.RandomState(0)
    n, d = 12, 2
    dims = [1, 2, 4, 8, 8, 8, 8, 8, 8, 8, 4, 2, 1]
    arrays = [rng.standard_normal((dims[i], d, dims[i + 1])) for i in range(n)]
    mps = tg.MatrixProductState(arrays, device="cpu")
    path = tmp_path / "state.npz"
    mps.save(str(path))
    f = np.load(str(path))
    assert list(f.files) == [f"I{s}" for s in range(n)]
    assert f["I0"].shape == (d, 2) and f[f"I{n - 1}"].shape == (2, d) and f["I5"].shape == (8, d, 8)
    back = tg.MatrixProductState.load(str(path), device="cpu")
    for a, b in zip(arrays, back.tensors):
        np.testing.assert_array_equal(a, b.numpy())
    # a reference-written file: site tags in site order, boundary tensors 2-index
    ref = tmp_path / "ref.npz"
    np.savez(str(ref), **{f"I{s}": (a[0] if s == 0 else a[:, :, 0] if s == n - 1 else a) for s, a in enumerate(arrays)})
    back2 = tg.MatrixProductState.load(str(ref), device="cpu")
    for a, b in zip(arrays, back2.tensors):
        np.testing.assert_array_equal(a, b.numpy())
    with pytest.raises(ValueError):
        mps.save(str(tmp_path / "state.txt"))
    with pytest.raises(ValueError):
        tg.MatrixProductState.load(str(tmp_path / "state.hdf"))
