"""The allocation-free one-site matvec (tnx_matvec1_noalloc) against the oracle.

Callers that cannot allocate device memory where they need H_eff x (a stream capture that
must not allocate, host bindings without a device allocator) use tnx_matvec1_noalloc, whose
scratch is a static device array inside libtnx. Its results are checked against the CPU
oracle's one-site matvec (an independent restatement of the reference contraction) and
against the workspace entry point tnx_matvec1, on two calls in a row, because every call
shares the array and the second call must not see the first one's leftovers. This file is
collected last so that a failure here comes after every other test has run; it also passes
on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import mps as omps

pytestmark = pytest.mark.gpu


def _lib():
    import tnpy_gb300._lib as L

    f = L.lib.tnx_matvec1_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int64] * 5 + [ctypes.c_void_p]
    return L


def _case(seed, chi_l, chi_r):
    rng = np.random.RandomState(seed)
    return (rng.standard_normal((chi_l, 5, chi_l)), rng.standard_normal((5, 5, 2, 2)),
            rng.standard_normal((chi_r, 5, chi_r)), rng.standard_normal((chi_l, 2, chi_r)))


def _dev(arrays, dev):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


def test_noalloc_matches_oracle_and_workspace_entry_point(cuda):
    L = _lib()
    import tnpy_gb300.kernels as K

    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row: the static scratch keeps the first call's contents
    for seed, (chi_l, chi_r) in enumerate([(96, 128), (200, 64)]):
        host = _case(seed, chi_l, chi_r)
        Lt, Wt, Rt, xt = _dev(host, cuda)
        y = torch.full((chi_l, 2, chi_r), float("nan"), dtype=torch.float64, device=cuda)
        st = L.lib.tnx_matvec1_noalloc(Lt.data_ptr(), Wt.data_ptr(), Rt.data_ptr(), xt.data_ptr(), y.data_ptr(),
                                       chi_l, 2, chi_r, 5, 5, stream)
        assert st == L.TNX_OK, L.lib.tnx_last_error()
        ref_ws = K.matvec1(Lt, Wt, Rt, xt, precision="fp64").cpu().numpy()
        got = y.cpu().numpy()
        ref = omps.one_site_matvec(*host)
        # FP64 contraction against the oracle: 1e-12 relative to the largest entry
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
        np.testing.assert_allclose(got, ref_ws, rtol=1e-12, atol=1e-12 * np.abs(ref_ws).max())


def test_noalloc_rejects_oversized_problem(cuda):
    L = _lib()
    Lt, Wt, Rt, xt = _dev(_case(3, 8, 8), cuda)
    # chi = 1024 would need 10.5M elements per intermediate: rejected before any launch
    st = L.lib.tnx_matvec1_noalloc(Lt.data_ptr(), Wt.data_ptr(), Rt.data_ptr(), xt.data_ptr(), xt.data_ptr(),
                                   1024, 2, 1024, 5, 5, torch.cuda.current_stream().cuda_stream)
    assert st == L.TNX_ERR_SHAPE
    assert b"static scratch" in L.lib.tnx_last_error()
