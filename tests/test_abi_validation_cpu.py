"""Error behaviour of the C ABI without a GPU: every entry point checks its arguments before it
touches the device, so invalid calls return their status code (and a message) on any host.
Pointers are placeholders: no call below gets past its failing check."""
import ctypes

import pytest
import torch

import tnpy_gb300._lib as L

P = 16  # non-null placeholder address, never dereferenced by a call that fails validation


def _err():
    return L.lib.tnx_last_error().decode()


def test_qr_rejects_wide_and_empty():
    assert L.lib.tnx_qr(P, 4, 8, P, P, None, 0, None) == L.TNX_ERR_SHAPE
    assert "m >= n" in _err()
    assert L.lib.tnx_qr(P, 0, 0, P, P, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_qr(None, 4, 4, P, P, None, 0, None) == L.TNX_ERR_INVALID_ARG


def test_gauge_move_rejects_bad_arguments():
    # precision, direction, sizes, and a split bond larger than the fused dimension
    assert L.lib.tnx_gauge_move(1, P, P, 4, 2, 4, 4, 9, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_gauge_move(2, P, P, 4, 2, 4, 4, 0, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_gauge_move(1, P, P, 0, 2, 4, 4, 0, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_gauge_move(1, P, P, 2, 2, 8, 4, 0, None, 0, None) == L.TNX_ERR_SHAPE
    assert L.lib.tnx_gauge_move(-1, P, P, 8, 2, 2, 4, 0, None, 0, None) == L.TNX_ERR_SHAPE


@pytest.mark.parametrize("max_iter,max_basis,tol,precision,expect", [
    (0, 24, 1e-8, 0, L.TNX_ERR_INVALID_ARG),      # no matvec allowed
    (100, 1, 1e-8, 0, L.TNX_ERR_INVALID_ARG),     # basis below 2
    (100, 65, 1e-8, 0, L.TNX_ERR_INVALID_ARG),    # basis above the kernels' 64
    (100, 24, -1.0, 0, L.TNX_ERR_INVALID_ARG),    # negative tolerance
    (100, 24, 1e-8, 3, L.TNX_ERR_INVALID_ARG),    # unknown precision
])
def test_davidson_rejects_bad_arguments(max_iter, max_basis, tol, precision, expect):
    ev, rn, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    st = L.lib.tnx_davidson1(P, P, P, P, 4, 2, 4, 5, 5, tol, max_iter, max_basis, precision, ctypes.byref(ev),
                             ctypes.byref(rn), ctypes.byref(it), None, 0, None)
    assert st == expect, _err()


def test_davidson_rejects_large_mpo_bond():
    ev, rn, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    st = L.lib.tnx_davidson1(P, P, P, P, 4, 2, 4, 33, 5, 1e-8, 100, 24, 0, ctypes.byref(ev), ctypes.byref(rn),
                             ctypes.byref(it), None, 0, None)
    assert st == L.TNX_ERR_SHAPE


def test_gemm_oz_rejects_negative_size():
    st = L.lib.tnx_gemm_oz(0, 0, -1, 4, 4, 1.0, P, 4, P, 4, 0.0, P, 4, None, 0, None)
    assert st == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_gemm_oz(0, 0, 4, 4, 4, 1.0, None, 4, P, 4, 0.0, P, 4, None, 0, None) == L.TNX_ERR_INVALID_ARG


def test_gauge_move_bad_direction_raises_keyerror():
    """The Python mirror raises the reference's exception for a direction that is neither
    left nor right (MatrixProductState.split_tensor, matrix_product_state.py:187-225)."""
    import tnpy_gb300.kernels as K

    a = torch.zeros((4, 2, 4), dtype=torch.float64)
    nb = torch.zeros((4, 2, 4), dtype=torch.float64)
    with pytest.raises(KeyError):
        K.gauge_move(0, a, nb)


@pytest.mark.parametrize("chi_l,d,chi_r,dl,dr", [
    (2**40, 2, 2**40, 5, 5),          # the product of the bonds alone would wrap int64
    (2**62, 2, 3, 5, 5),              # one huge bond
    (2**21 + 1, 2, 1, 5, 5),          # one bond just above the static scratch
    (8, 2**40, 8, 1, 1),              # a physical dimension that would wrap the product
])
def test_noalloc_matvec_rejects_sizes_that_would_overflow(chi_l, d, chi_r, dl, dr):
    f = L.lib.tnx_matvec1_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int64] * 5 + [ctypes.c_void_p]
    st = f(P, P, P, P, P, chi_l, d, chi_r, dl, dr, None)
    assert st == L.TNX_ERR_SHAPE, _err()


def test_gemm_oz_batched_rejects_bad_arguments():
    f = L.lib.tnx_gemm_oz_batched
    assert f(0, 0, -1, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0, P, 4, 16, 2, 1, None, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert f(0, 0, 4, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0, P, 4, 16, 0, 1, None, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert f(0, 0, 4, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0, P, 4, 16, 2, 0, None, None, 0, None) == L.TNX_ERR_INVALID_ARG
    assert f(0, 0, 4, 4, 4, 1.0, None, 4, 16, P, 4, 16, 0.0, P, 4, 16, 2, 1, None, None, 0, None) == \
        L.TNX_ERR_INVALID_ARG
    # one launch covers batch x split CTAs layers: at most 65535
    assert f(0, 0, 4, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0, P, 4, 16, 40000, 2, None, None, 0, None) == \
        L.TNX_ERR_INVALID_ARG
    assert "split" in _err()


def test_eigh_batched_df64_rejects_bad_arguments():
    f = L.lib.tnx_eigh_batched_df64
    assert f(P, P, P, 2, 65, 4, P, P, None) == L.TNX_ERR_SHAPE      # matrices above 64 rows
    assert "64" in _err()
    assert f(P, P, P, 2, 16, 17, P, P, None) == L.TNX_ERR_INVALID_ARG  # keep above max_size
    assert f(None, P, P, 2, 16, 4, P, P, None) == L.TNX_ERR_INVALID_ARG
    assert f(P, P, P, 0, 16, 4, P, P, None) == L.TNX_OK             # empty batch: nothing to do


def test_davidson_ex_rejects_unknown_flags():
    ev, rn, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    st = L.lib.tnx_davidson1_ex(P, P, P, P, 4, 2, 4, 5, 5, 1e-8, 100, 24, 1, 2, ctypes.byref(ev), ctypes.byref(rn),
                                ctypes.byref(it), None, 0, None)
    assert st == L.TNX_ERR_INVALID_ARG and "flags" in _err()


def test_profiler_families():
    # families 0..7 (7: the Ozaki GEMM's narrow products); an empty window ends with no launches
    for fam in range(8):
        assert L.lib.tnx_profile_begin(fam) == L.TNX_OK
        n, ms, fl, by = ctypes.c_int(-1), ctypes.c_double(-1), ctypes.c_double(-1), ctypes.c_double(-1)
        assert L.lib.tnx_profile_end(ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by)) == L.TNX_OK
        assert (n.value, ms.value, fl.value, by.value) == (0, 0.0, 0.0, 0.0)
    assert L.lib.tnx_profile_begin(8) == L.TNX_ERR_INVALID_ARG
    assert L.lib.tnx_profile_begin(-1) == L.TNX_ERR_INVALID_ARG
