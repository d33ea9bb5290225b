"""Control of the library's autotuner (include/tnx.h, autotune.cu).

The first call of each GEMM shape times its candidate kernels (double-FP32 GEMM tile, FP64-class
engine: tcgen05 Ozaki or double-FP32 SIMT, split-BF16 tcgen05 tile) and every later call of that
shape uses the fastest. ``choices()`` lists what was picked, for reports and benchmarks.
"""
from __future__ import annotations

import ctypes

from ._lib import check, lib

KINDS = {1: "df64_gemm_tile", 2: "fp64_class_engine", 3: "bf16x3_gemm_tile"}
VARIANTS = {1: ["64x128/256thr", "32x32/64thr"], 2: ["ozaki_tcgen05", "df64_simt"], 3: ["128x256", "128x128"]}


def enable(on: bool = True) -> None:
    check("tnx_autotune_set", lib.tnx_autotune_set(1 if on else 0))


def clear() -> None:
    check("tnx_autotune_clear", lib.tnx_autotune_clear())


def count() -> int:
    return int(lib.tnx_autotune_count())


def choices() -> list[dict]:
    """One dict per tuned shape: kind, key (the shape numbers), chosen variant and the measured
    milliseconds of every candidate (-1 for a candidate that did not apply)."""
    n = lib.tnx_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(int(n))
    lib.tnx_autotune_report(buf, n)
    out = []
    for line in buf.value.decode().splitlines():
        head, tail = line.split("->")
        key = [int(x) for x in head.split()]
        vals = tail.split()
        kind, choice = key[0], int(vals[0])
        out.append({"kind": KINDS.get(kind, str(kind)), "key": key[1:], "choice": VARIANTS.get(kind, [])[choice]
                    if choice < len(VARIANTS.get(kind, [])) else choice, "ms": [float(v) for v in vals[1:]]})
    return out
