"""Small fixed workloads for profiling single kernels (e.g. under ncu).

    python -m tnpy_gb300.prof matvec --chi 1024      # split-BF16 tcgen05 matvec (+ FP64-class env)
    python -m tnpy_gb300.prof env --chi 1024         # double-FP32 environment update
    python -m tnpy_gb300.prof qr --m 2048 --n 1024   # Householder QR (cluster panel), FP64 GEMMs
    python -m tnpy_gb300.prof gauge --chi 1024       # one-site gauge move (QR with double-FP32 GEMMs)
    python -m tnpy_gb300.prof davidson --chi 512     # one mixed-precision local eigensolve
    python -m tnpy_gb300.prof sweep --chi 1024 --sites 100   # fDMRG sweeps of XXZ(n, -0.5), per family
    python -m tnpy_gb300.prof tsdrg --sites 128 --chi 32 --batch 64 [--precision mixed]   # batched tSDRG
    python -m tnpy_gb300.prof chains --sites 64 --chi 64 --batch 64   # lockstep fDMRG chains, one sweep
    python -m tnpy_gb300.prof svd --m 2048 --n 1024   # one-sided Jacobi SVD
    python -m tnpy_gb300.prof ed --sites 12           # dense MPO Hamiltonian + full spectrum

Each mode runs two warm-up calls and then --reps calls of the same shapes, on random seeded
inputs, and prints the CUDA-event time per call and its split over the library's kernel
families (tnx_profile_begin / tnx_profile_end).
"""
from __future__ import annotations

import argparse
import ctypes

import torch

from . import kernels as K
from ._lib import lib

FAMILIES = ["tcgen05 GEMM", "FP64-class GEMM", "vector", "QR panel", "eigh", "other", "Ozaki GEMM",
            "Ozaki GEMM (narrow)"]


def _families(fn, reps):
    """Per-family device time of `reps` calls (ms per call), from the library's event profiler."""
    out = {}
    for fam, name in enumerate(FAMILIES):
        torch.cuda.synchronize()
        lib.tnx_profile_begin(fam)
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        n, ms, fl, by = ctypes.c_int(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        lib.tnx_profile_end(ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(by))
        if n.value:
            out[name] = (n.value / reps, ms.value / reps)
    return out


def _time(fn, reps):
    fn()
    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def _fmt(fam):
    return ", ".join(f"{k}: {n:.0f} launches {ms:.2f} ms" for k, (n, ms) in fam.items())


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("mode", choices=["matvec", "env", "qr", "gauge", "davidson", "sweep", "tsdrg", "chains", "svd",
                                    "ed"])
    p.add_argument("--batch", type=int, default=64)
    p.add_argument("--no-families", action="store_true", help="skip the per-family profiled repetitions")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"], help="tsdrg mode's precision")
    p.add_argument("--sites", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--chi", type=int, default=1024)
    p.add_argument("--m", type=int, default=2048)
    p.add_argument("--n", type=int, default=1024)
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args(argv)
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cpu").manual_seed(0)
    rnd = lambda *shape: torch.randn(*shape, generator=g, dtype=torch.float64).to(dev)  # noqa: E731
    chi = a.chi
    if a.mode == "sweep":
        import tnpy_gb300 as tg

        f = tg.FiniteDMRG(tg.model.XXZ(a.sites, -0.5).mpo, bond_dim=chi, precision="mixed", seed=1234,
                          compute_variance=False, device=dev)
        dirs = [tg.Direction.RIGHTWARD, tg.Direction.LEFTWARD]
        step = [0]

        def sweep():
            f.sweep(dirs[step[0] % 2], tol=1e-8)
            step[0] += 1

        for _ in range(a.warmup):
            sweep()
        t = _time(sweep, a.reps)
        fam = {} if a.no_families else _families(sweep, 1)
        print(f"sweep XXZ({a.sites}) chi={chi}: {t:.1f} ms per sweep; one sweep per family: " + _fmt(fam))
        # one more sweep inside an NVTX range: `ncu --nvtx --nvtx-include "profiled sweep/"` captures
        # exactly its launches
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("profiled sweep")
        sweep()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        return
    if a.mode == "tsdrg":
        import tnpy_gb300 as tg

        mpos = [tg.model.RandomCouplingHeisenberg(a.sites, delta=1.0, h=0.0, seed=r).mpo for r in range(a.batch)]

        def run():
            tg.BatchedTSDRG(mpos, chi=chi, precision=a.precision).run()

        t = _time(run, a.reps)
        print(f"tsdrg n={a.sites} chi={chi} x{a.batch} {a.precision}: {t:.1f} ms per batch "
              f"({a.batch / t * 1e3:.1f} realisations/s)")
        return
    if a.mode == "chains":
        import tnpy_gb300 as tg

        mpos = [tg.model.RandomHeisenberg(a.sites, h=1.0, seed=100 + c).mpo for c in range(a.batch)]
        b = tg.BatchedFiniteDMRG(mpos, bond_dim=chi, seed=100, precision="mixed", device=dev)
        dirs = [tg.Direction.RIGHTWARD, tg.Direction.LEFTWARD]
        step = [0]

        def sweep():
            b.sweep(dirs[step[0] % 2], tol=1e-8)
            step[0] += 1

        for _ in range(a.warmup):
            sweep()
        t = _time(sweep, a.reps)
        print(f"chains n={a.sites} chi={chi} x{a.batch}: {t:.1f} ms per lockstep sweep")
        return
    if a.mode == "svd":
        m = rnd(a.m, a.n)
        t = _time(lambda: K.svd(m), a.reps)
        print(f"svd {a.m}x{a.n}: {t:.3f} ms")
        return
    if a.mode == "ed":
        import tnpy_gb300 as tg

        mpo = tg.model.RandomHeisenberg(a.sites, h=0.5, seed=1).mpo
        t = _time(lambda: tg.ExactDiagonalization(mpo, device=dev), a.reps)
        print(f"exact diagonalisation n={a.sites}: {t:.1f} ms")
        return
    if a.mode in ("matvec", "env", "davidson"):
        L, R, W, x = rnd(chi, 5, chi), rnd(chi, 5, chi), rnd(5, 5, 2, 2), rnd(chi, 2, chi)
        L = 0.5 * (L + L.permute(2, 1, 0))
        R = 0.5 * (R + R.permute(2, 1, 0))
        W = 0.5 * (W + W.permute(0, 1, 3, 2))
        L, R, W = L.contiguous(), R.contiguous(), W.contiguous()
    if a.mode == "matvec":
        t = _time(lambda: K.matvec1(L, W, R, x, precision="mixed"), a.reps)
        flops = 40 * chi**3 + 200 * chi**2
        print(f"matvec mixed chi={chi}: {t:.3f} ms, {flops / t / 1e9:.1f} TFLOP/s algorithmic")
    elif a.mode == "env":
        t = _time(lambda: K.env_update(1, L, x, W, precision="df64"), a.reps)
        print(f"env update df64 chi={chi}: {t:.3f} ms")
    elif a.mode == "qr":
        m = rnd(a.m, a.n)
        fn = lambda: K.qr(m)  # noqa: E731
        t = _time(fn, a.reps)
        print(f"qr {a.m}x{a.n}: {t:.3f} ms  " + _fmt(_families(fn, a.reps)))
    elif a.mode == "gauge":
        site, nb = rnd(chi, 2, chi), rnd(chi, 2, chi)

        def fn():
            K.gauge_move(1, site.clone(), nb.clone(), precision="mixed")

        t = _time(fn, a.reps)
        print(f"gauge move df64 chi={chi}: {t:.3f} ms  " + ("" if a.no_families else _fmt(_families(fn, a.reps))))
    else:
        stats = {}

        def solve():
            y = x.clone()
            stats["out"] = K.davidson1(L, W, R, y, tol=1e-8, precision="mixed")

        t = _time(solve, a.reps)
        e, rn, its, ok = stats["out"]
        print(f"davidson mixed chi={chi}: {t:.3f} ms, {its} matvecs, residual {rn:.2e}, converged {ok}  "
              + _fmt(_families(solve, a.reps)))


if __name__ == "__main__":
    main()
