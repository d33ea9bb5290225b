"""ctypes binding of libtnx.so (the C ABI declared in include/tnx.h).

The library is required: importing this module on a machine where it has not
been built raises ImportError, and every wrapper raises if its tensors are not
contiguous FP64 CUDA tensors. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

import torch

_PKG = Path(__file__).resolve().parent
_LIB_PATH = Path(os.environ.get("TNX_LIB", _PKG / "libtnx.so"))

TNX_OK = 0
TNX_ERR_INVALID_ARG = 1
TNX_ERR_SHAPE = 2
TNX_ERR_WORKSPACE = 3
TNX_ERR_NOT_CONVERGED = 4
TNX_ERR_CUDA = 5
TNX_ERR_TIMEOUT = 6
TNX_ERR_UNSUPPORTED = 7

FP64 = 0
BF16X3 = 1
DF64 = 2
PRECISIONS = {"fp64": FP64, "mixed": BF16X3, "bf16x3": BF16X3, "df64": DF64}

if not _LIB_PATH.exists():
    raise ImportError(
        f"{_LIB_PATH} is missing: build the CUDA library first "
        "(python -c 'import __graft_entry__ as g; g.build()' or python tnpy_gb300/build.py)"
    )

lib = ctypes.CDLL(str(_LIB_PATH))

_c = ctypes
_i64, _int, _dbl, _vp, _sz = _c.c_int64, _c.c_int, _c.c_double, _c.c_void_p, _c.c_size_t
_pi = _c.POINTER(_c.c_int)
_pd = _c.POINTER(_c.c_double)

SIGNATURES = {
    "tnx_status_string": (_c.c_char_p, [_int]),
    "tnx_last_error": (_c.c_char_p, []),
    "tnx_version": (_int, []),
    "tnx_device_ok": (_int, []),
    "tnx_launch_count": (_c.c_longlong, []),
    "tnx_profile_begin": (_int, [_int]),
    "tnx_profile_end": (_int, [_pi, _pd, _pd, _pd]),
    "tnx_matvec1_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _int]),
    "tnx_matvec1": (_int, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _int, _vp, _sz, _vp]),
    "tnx_full_matrix1": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _vp]),
    "tnx_diag1": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _vp]),
    "tnx_env_update_workspace_bytes": (_sz, [_int, _i64, _i64, _i64, _i64, _i64, _int]),
    "tnx_env_update": (_int, [_int, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _int, _vp, _sz, _vp]),
    "tnx_davidson1_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _int, _int]),
    "tnx_davidson1": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _dbl, _int, _int, _int,
                             _pd, _pd, _pi, _vp, _sz, _vp]),
    "tnx_davidson1_ex": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _dbl, _int, _int, _int, _int,
                                _pd, _pd, _pi, _vp, _sz, _vp]),
    "tnx_davidson1_stats": (_int, [_pi]),
    "tnx_gdavidson1_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _i64, _i64, _int]),
    "tnx_gdavidson1": (_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _i64, _i64, _dbl,
                              _int, _int, _int, _pd, _pd, _pi, _vp, _sz, _vp]),
    "tnx_mpo_apply_site": (_int, [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _vp]),
    "tnx_eigh_batched_workspace_bytes": (_sz, [_int, _int, _int]),
    "tnx_eigh_batched": (_int, [_vp, _vp, _vp, _int, _int, _int, _vp, _vp, _vp, _sz, _vp]),
    "tnx_eigh_batched_df64": (_int, [_vp, _vp, _vp, _int, _int, _int, _vp, _vp, _vp]),
    "tnx_qr_workspace_bytes": (_sz, [_i64, _i64]),
    "tnx_qr": (_int, [_vp, _i64, _i64, _vp, _vp, _vp, _sz, _vp]),
    "tnx_gauge_move_workspace_bytes": (_sz, [_int, _i64, _i64, _i64, _i64]),
    "tnx_gauge_move": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _i64, _int, _vp, _sz, _vp]),
    "tnx_gemm_df64": (_int, [_int, _int, _i64, _i64, _i64, _dbl, _vp, _i64, _vp, _i64, _dbl, _vp, _i64, _vp]),
    "tnx_gemm_oz_workspace_bytes": (_sz, [_i64, _i64, _i64]),
    "tnx_gemm_oz": (_int, [_int, _int, _i64, _i64, _i64, _dbl, _vp, _i64, _vp, _i64, _dbl, _vp, _i64, _vp, _sz,
                           _vp]),
    "tnx_gemm_oz_batched_workspace_bytes": (_sz, [_i64, _i64, _i64, _int, _int]),
    "tnx_gemm_oz_batched": (_int, [_int, _int, _i64, _i64, _i64, _dbl, _vp, _i64, _i64, _vp, _i64, _i64, _dbl, _vp,
                                   _i64, _i64, _int, _int, _vp, _vp, _sz, _vp]),
    "tnx_gemm_bf16x3_workspace_bytes": (_sz, [_i64, _i64, _i64]),
    "tnx_gemm_bf16x3": (_int, [_i64, _i64, _i64, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tnx_tsdrg_block_hamiltonian": (_int, [_vp, _vp, _vp, _int, _vp, _vp, _int, _int, _vp]),
    "tnx_tsdrg_project": (_int, [_vp, _vp, _vp, _vp, _int, _vp, _int, _int, _int, _int, _vp]),
    "tnx_tsdrg_block_eigh_workspace_bytes": (_sz, [_int, _int, _int, _int]),
    "tnx_tsdrg_block_eigh": (_int, [_vp, _vp, _vp, _int, _int, _int, _int, _int, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tnx_batched_matvec1_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _int]),
    "tnx_batched_matvec1": (_int, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _int, _i64, _i64, _i64,
                                   _i64, _i64, _int, _vp, _sz, _vp]),
    "tnx_batched_full_matrix1": (_int, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _int, _i64, _i64, _i64, _i64, _i64,
                                        _vp]),
    "tnx_batched_env_update_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _int]),
    "tnx_batched_env_update": (_int, [_int, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _int, _i64, _i64, _i64,
                                      _i64, _i64, _int, _vp, _sz, _vp]),
    "tnx_batched_davidson1_workspace_bytes": (_sz, [_i64, _i64, _i64, _i64, _i64, _int, _int]),
    "tnx_batched_davidson1": (_int, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _int, _i64, _i64, _i64, _i64,
                                     _i64, _dbl, _int, _int, _int, _vp, _vp, _pi, _vp, _vp, _sz, _vp]),
    "tnx_batched_gauge_move_workspace_bytes": (_sz, [_int, _i64, _i64, _i64, _i64, _int]),
    "tnx_batched_gauge_move": (_int, [_int, _vp, _i64, _vp, _i64, _int, _i64, _i64, _i64, _i64, _int, _vp, _sz,
                                      _vp]),
    "tnx_full_hamiltonian": (_int, [_vp, _int, _int, _int, _vp, _vp]),
    "tnx_shift_to_spd": (_int, [_vp, _i64, _vp, _int, _vp]),
    "tnx_autotune_set": (_int, [_int]),
    "tnx_autotune_clear": (_int, []),
    "tnx_autotune_count": (_int, []),
    "tnx_autotune_report": (_sz, [_c.c_char_p, _sz]),
    "tnx_svd_workspace_bytes": (_sz, [_i64, _i64, _int]),
    "tnx_svd": (_int, [_vp, _i64, _i64, _vp, _vp, _vp, _pi, _vp, _sz, _vp]),
    "tnx_gemm_f64": (_int, [_int, _int, _i64, _i64, _i64, _dbl, _vp, _i64, _i64, _vp, _i64, _i64, _dbl,
                            _vp, _i64, _i64, _i64, _vp]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args


class TnxError(RuntimeError):
    def __init__(self, name: str, status: int):
        msg = lib.tnx_last_error().decode(errors="replace")
        super().__init__(f"{name}: {lib.tnx_status_string(status).decode()} ({status}): {msg}")
        self.status = status


class NotConverged(TnxError):
    pass


def check(name: str, status: int):
    if status == TNX_OK:
        return
    if status in (TNX_ERR_INVALID_ARG, TNX_ERR_SHAPE):
        raise ValueError(TnxError(name, status).args[0])
    if status == TNX_ERR_UNSUPPORTED:
        raise NotImplementedError(TnxError(name, status).args[0])
    if status == TNX_ERR_NOT_CONVERGED:
        raise NotConverged(name, status)
    raise TnxError(name, status)


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a contiguous FP64 (or index) CUDA tensor."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("tnx expects CUDA tensors (there is no CPU path)")
    if not t.is_contiguous():
        raise ValueError("tnx expects contiguous tensors")
    return t.data_ptr()


def stream_ptr(stream: torch.cuda.Stream | None = None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Workspace:
    """Scratch buffer per (device, stream), grown on demand (torch caching allocator).

    Library calls on different streams must not share scratch, so host threads that drive
    independent chains on their own streams (``BatchedFiniteDMRG``) each get their own buffer;
    the buffer is allocated while its stream is current, so the caching allocator orders its
    reuse on that stream."""

    _bufs: dict[tuple[int, int], torch.Tensor] = {}
    _lock = threading.Lock()

    @classmethod
    def get(cls, nbytes: int, device: torch.device) -> tuple[int, int]:
        idx = device.index if device.index is not None else torch.cuda.current_device()
        key = (idx, torch.cuda.current_stream(idx).cuda_stream)
        with cls._lock:
            buf = cls._bufs.get(key)
            if buf is None or buf.numel() < nbytes:
                if buf is not None:
                    del cls._bufs[key]
                    del buf
                size = max(int(nbytes * 1.25), 1 << 20)
                buf = torch.empty(size, dtype=torch.uint8, device=torch.device("cuda", idx))
                cls._bufs[key] = buf
            return buf.data_ptr(), buf.numel()
