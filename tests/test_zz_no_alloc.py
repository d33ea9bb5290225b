"""The allocation-free one-site matvec (tnx_matvec1_noalloc) against the workspace entry point.

Callers that cannot allocate device memory where they need H_eff x (a stream capture that
must not allocate, host bindings without a device allocator) use tnx_matvec1_noalloc, whose
scratch is a static device array inside libtnx. This file is collected last so that a failure
here comes after every other test has run; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    import tnpy_gb300._lib as L

    f = L.lib.tnx_matvec1_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int64] * 5 + [ctypes.c_void_p]
    return L


def _case(seed, chi_l, chi_r, dev):
    rng = np.random.RandomState(seed)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    return (t(rng.standard_normal((chi_l, 5, chi_l))), t(rng.standard_normal((5, 5, 2, 2))),
            t(rng.standard_normal((chi_r, 5, chi_r))), t(rng.standard_normal((chi_l, 2, chi_r))))


def test_noalloc_matches_workspace_entry_point(cuda):
    L = _lib()
    import tnpy_gb300.kernels as K

    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row: the static scratch keeps the first call's contents
    for seed, (chi_l, chi_r) in enumerate([(96, 128), (200, 64)]):
        Lt, Wt, Rt, xt = _case(seed, chi_l, chi_r, cuda)
        y = torch.empty((chi_l, 2, chi_r), dtype=torch.float64, device=cuda)
        st = L.lib.tnx_matvec1_noalloc(Lt.data_ptr(), Wt.data_ptr(), Rt.data_ptr(), xt.data_ptr(), y.data_ptr(),
                                       chi_l, 2, chi_r, 5, 5, stream)
        assert st == L.TNX_OK, L.lib.tnx_last_error()
        ref = K.matvec1(Lt, Wt, Rt, xt, precision="fp64")
        torch.cuda.synchronize()
        np.testing.assert_allclose(y.cpu().numpy(), ref.cpu().numpy(), rtol=1e-12,
                                   atol=1e-12 * ref.abs().max().item())


def test_noalloc_rejects_oversized_problem(cuda):
    L = _lib()
    Lt, Wt, Rt, xt = _case(3, 8, 8, cuda)
    # chi = 1024 would need 10.5M elements per intermediate: rejected before any launch
    st = L.lib.tnx_matvec1_noalloc(Lt.data_ptr(), Wt.data_ptr(), Rt.data_ptr(), xt.data_ptr(), xt.data_ptr(),
                                   1024, 2, 1024, 5, 5, torch.cuda.current_stream().cuda_stream)
    assert st == L.TNX_ERR_SHAPE
    assert b"static scratch" in L.lib.tnx_last_error()
