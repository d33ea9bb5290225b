#!/usr/bin/env python
"""Benchmark: one-site fDMRG sweeps of the XXZ chain on GB300 (sweeps/s), plus the CPU
restatement of the reference path timed on the host cores.

A step is one full sweep (n-1 site updates: lowest eigenpair of the one-site effective
Hamiltonian, 1e-5 perturbation, gauge move, environment update) of XXZ(n, delta=-0.5),
i.e. H = sum SxSx + SySy + 0.5 SzSz, at fixed bond dimension chi, starting from a seeded
random MPS. Environments (n * 2 * chi^2 * 5 * 8 bytes, 8.4 GB at n=100, chi=1024) are
far larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--n 100] [--chi 1024] [--precision mixed|fp64]

Under torchrun every rank runs an independent chain (replicas; a sweep does not shard),
value = total sweeps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "DMRG sweep s & matvec TFLOP/s, mixed vs FP64 GPU at |dE|<=1e-9; tSDRG realiz/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=100)
    p.add_argument("--chi", type=int, default=1024)
    p.add_argument("--delta", type=float, default=-0.5)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--tol", type=float, default=1e-8)
    p.add_argument("--seed", type=int, default=1234)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the matvec-form and tSDRG measurements")
    p.add_argument("--tsdrg-realizations", type=int, default=1024)
    p.add_argument("--chains", type=int, default=256, help="independent chi=64 chains of the batched fDMRG line")
    return p.parse_args()


def workload(a):
    return {"workload": f"fdmrg_onesite_xxz_n{a.n}_chi{a.chi}_{a.precision}", "model": "XXZ(n, delta=-0.5)",
            "n": a.n, "chi": a.chi, "d": 2, "mpo_bond": 5, "precision": a.precision, "tol": a.tol,
            "seed": a.seed, "step": "one full sweep (n-1 site updates)", "l2": "inputs > L2 (no flush)",
            "parallelism": f"replicas{a.gpus}"}


# ------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(gpu_index)], stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU restatement (oracle)
def sweep_site_weight(n: int, chi: int, d: int = 2) -> float:
    """Sum over the n-1 site updates of one sweep of chi_l chi_r max(chi_l, chi_r) / chi^3: the
    number of full-chi site updates a sweep's work equals (the matvec, environment update and
    gauge move of a site scale with that product; 81.1 for n=100, chi=1024, where 80 of the 99
    sites have full bonds)."""
    from oracle import mps as omps

    dims = omps.bond_dims(n, chi, d)
    return sum(dims[i] * dims[i + 1] * max(dims[i], dims[i + 1]) for i in range(n - 1)) / float(chi) ** 3


class CpuBulkPair:
    """Two neighbouring bulk sites i, i+1 of a chain in the CPU restatement, with the centre on
    site i: L_i, R_{i+1} fixed, the two site tensors and their MPO tensors. ``step`` performs one
    site update of FiniteDMRG.sweep (tnpy/finite_dmrg.py:143-171) in numpy: the lowest eigenpair
    from the current site tensor (oracle.eigsh_gd, the GD+1 restatement of primme.eigsh, at the
    sweep's tol), the 1e-5 perturbation, the SVD gauge move onto the neighbour and the
    environment update; the updates alternate rightward at i and leftward at i+1, i.e. a sweep
    bouncing between the two sites."""

    def __init__(self, L, Wi, Wj, R, ai, aj, tol):
        from oracle import mps as omps

        self.L, self.Wi, self.Wj, self.R = L, Wi, Wj, R
        self.ai, self.aj = ai, aj
        self.tol = tol
        self.Ri = omps.update_right(R, aj, Wj)  # R_i for the first (rightward) update at i
        self.Lj = None
        self.right = True
        self.matvecs = 0
        self.energy = None

    def step(self, tol: float | None = None):
        from oracle import eigsh_gd
        from oracle import mps as omps

        if self.right:
            L, W, R, x = self.L, self.Wi, self.Ri, self.ai
        else:
            L, W, R, x = self.Lj, self.Wj, self.R, self.aj
        shape = x.shape
        e, v, mv, _ = eigsh_gd.eigsh_gd(lambda u: omps.one_site_matvec(L, W, R, u.reshape(shape)).reshape(-1),
                                        x, tol=self.tol if tol is None else tol)
        psi = v.reshape(shape)
        psi = psi + 1e-5 * omps.one_site_matvec(L, W, R, psi)
        pair = [self.ai, self.aj]
        if self.right:
            pair[0] = psi
            omps.split_tensor(pair, 0, rightward=True)
            self.ai, self.aj = pair
            self.Lj = omps.update_left(self.L, self.ai, self.Wi)
        else:
            pair[1] = psi
            omps.split_tensor(pair, 1, rightward=False)
            self.ai, self.aj = pair
            self.Ri = omps.update_right(self.R, self.aj, self.Wj)
        self.right = not self.right
        self.matvecs += mv + 1
        self.energy = e
        return e, mv


def cpu_pair_from_random_mps(a):
    """A bulk pair with full chi on both sides, built in numpy from a seeded random MPS: the middle
    sites of XXZ(n_env, delta) with n_env = 2 ceil(log2 chi) + 2 (22 for chi = 1024), whose middle
    bonds reach chi, so that the local problem has the shape of every bulk site of the bench
    chain (L, R: chi x D x chi) while its environments take only ~n_env small contractions to
    build. Right-canonical tensors, centre moved from site 0 to the pair by QR."""
    import math

    import numpy as np

    from oracle import models as om
    from oracle import mps as omps

    half = max(1, math.ceil(math.log2(a.chi)))
    n = min(a.n, 2 * half + 2)
    i = n // 2 - 1
    W = om.uniform(om.xxz_mpo(n, a.delta))
    mps = omps.random_mps(n, a.chi, 2, seed=a.seed)
    for s in range(i):  # gauge the centre onto site i
        cl, d, cr = mps[s].shape
        q, r = np.linalg.qr(mps[s].reshape(cl * d, cr))
        mps[s] = q.reshape(cl, d, q.shape[1])
        mps[s + 1] = np.tensordot(r, mps[s + 1], axes=([1], [0]))
    L = np.ones((1, 1, 1))
    for s in range(i):
        L = omps.update_left(L, mps[s], W[s])
    R = np.ones((1, 1, 1))
    for s in range(n - 1, i + 1, -1):
        R = omps.update_right(R, mps[s], W[s])
    return L, W[i], W[i + 1], R, mps[i], mps[i + 1]


def cpu_site_updates(pair: "CpuBulkPair", steps: int, warmup: int, prepare_s: float = 0.0):
    """Per-step wall times of ``steps`` timed site updates after ``warmup`` untimed ones; with
    prepare_s > 0 the pair is first swept (untimed) until its energy settles to the pair's tol
    or prepare_s seconds pass, so that the timed updates see a converged state as the timed GPU
    sweeps do."""
    t_prep = time.perf_counter()
    prep = 0
    if prepare_s > 0:
        # loose local tolerance first (the random start is far from the pair's ground state),
        # then the sweep's tol until the energy settles
        last = None
        while time.perf_counter() - t_prep < prepare_s:
            loose = prep < 2
            e, _ = pair.step(tol=1e-5 if loose else None)
            prep += 1
            if not loose and last is not None and abs(e - last) < pair.tol * max(1.0, abs(e)):
                break
            last = e
    prep_s = time.perf_counter() - t_prep
    for _ in range(warmup):
        pair.step()
    mv0 = pair.matvecs
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        pair.step()
        times.append(time.perf_counter() - t0)
    return {"times": times, "matvecs_per_update": (pair.matvecs - mv0) / max(1, steps),
            "prepare_updates": prep, "prepare_s": prep_s}


def cpu_result(a, res, origin: str, kind: str = "port"):
    mean = statistics.fmean(res["times"])
    w = sweep_site_weight(a.n, a.chi)
    return {"value": 1.0 / (mean * w), "unit": "sweeps/s", "cores": os.cpu_count(), "kind": kind,
            "sample": f"{len(res['times'])} timed site updates (after the warm-up) of the numpy/scipy FP64 "
                      f"restatement bouncing between bulk sites {a.n // 2} and {a.n // 2 + 1} of XXZ(n={a.n}) at "
                      f"chi={a.chi}, {origin}; each: GD+1 eigensolver (primme restatement) at tol {a.tol:g} from the "
                      f"current site tensor, 1e-5 perturbation, SVD gauge move, environment update; "
                      f"sweep time = mean site update x {w:.1f} full-chi site equivalents of the {a.n - 1} sites",
            "seconds_per_site_update": mean, "site_updates_timed": len(res["times"]),
            "matvecs_per_site_update": res["matvecs_per_update"], "sweep_site_weight": w,
            "prepare_updates": res["prepare_updates"], "prepare_s": res["prepare_s"]}


# ------------------------------------------------------------------ secondary measurements
def matvec_forms(f, site: int):
    """Matvec TFLOP/s of the three arithmetic forms on the bench chain's own local operator at
    ``site`` (algorithmic flops 4 chi_l chi_r max(chi) D d + 2 chi_l chi_r D^2 d^2 per product),
    and the lowest local eigenvalue from the mixed and the FP64 Davidson on that operator."""
    import torch

    from tnpy_gb300 import kernels as K

    L, W, R = f.env.site_operator(site)
    x = f.mps.tensors[site].contiguous()
    cl, d, cr = x.shape
    D = W.shape[0]
    flops = 4.0 * cl * cr * max(cl, cr) * D * d + 2.0 * cl * cr * D * D * d * d
    out = {"site": site, "shape": [cl, d, cr], "flops_per_matvec": flops}
    for form, reps in (("mixed", 10), ("df64", 3), ("fp64", 2)):
        K.matvec1(L, W, R, x, precision=form)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            K.matvec1(L, W, R, x, precision=form)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[form] = {"ms": ms, "tflops": flops / (ms / 1e3) / 1e12}
    evs = {}
    for form in ("mixed", "fp64"):
        y = x.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e, rn, its, ok = K.davidson1(L, W, R, y, tol=1e-10, precision=form, max_iter=400)
        torch.cuda.synchronize()
        evs[form] = {"eval": e, "residual": rn, "matvecs": its, "converged": bool(ok),
                     "s": time.perf_counter() - t0}
    evs["local_dE_rel_mixed_vs_fp64"] = abs(evs["mixed"]["eval"] - evs["fp64"]["eval"]) / abs(evs["fp64"]["eval"])
    out["local_eigensolve"] = evs
    out["local_dE_rel_mixed_vs_fp64"] = abs(evs["mixed"]["eval"] - evs["fp64"]["eval"]) / abs(evs["fp64"]["eval"])
    return out


def fp64_sweep(f, direction, tol: float, mixed_s: float):
    """The plain FP64 GPU form against the mixed form on the same state: both chains start from a
    copy of the bench chain's current MPS (environments rebuilt in each form) and sweep once in
    the same direction; reports the FP64 sweep's seconds, the speed-up of the mixed form's timed
    sweeps over it, |dE|/|E| between the two energies after the sweep and the largest difference
    of the local <Sz_i> of the two states."""
    import torch

    import tnpy_gb300 as tg

    out, sz = {}, {}
    for form in ("fp64", "mixed"):
        mps = tg.MatrixProductState([t.clone() for t in f.mps.tensors], device=f.mps.device)
        g = tg.FiniteDMRG(f.env.mpo, bond_dim=f.bond_dim, mps=mps, precision=form, compute_variance=False,
                          device=f.mps.device)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = g.sweep(direction, tol=tol)
        torch.cuda.synchronize()
        out[form] = {"s": time.perf_counter() - t0, "energy": e,
                     "matvecs_per_site": g.stats["matvecs"] / max(1, g.stats["iterative_solves"]),
                     "unconverged": g.stats["unconverged"], "df64_retries": g.stats["df64_retries"]}
        sz[form] = tg.MatrixProductStateMeasurements(g.mps).local_sz()
        del g, mps
        torch.cuda.empty_cache()
    out["speedup_mixed_timed_vs_fp64"] = out["fp64"]["s"] / mixed_s
    out["dE_rel_mixed_vs_fp64"] = abs(out["mixed"]["energy"] - out["fp64"]["energy"]) / abs(out["fp64"]["energy"])
    out["max_sz_err_mixed_vs_fp64"] = float(abs(sz["mixed"] - sz["fp64"]).max())
    return out


def xxz_n32_line(with_cpu: bool):
    """Plain FP64 fDMRG of XXZ(32, delta=-0.5) (H = sum SxSx + SySy + 0.5 SzSz up to a sublattice
    rotation), chi=32, seeded random MPS, tol 1e-8, at most 10 sweeps: seconds per sweep on the
    GPU, the same run of the CPU restatement timed beside it, their final energies, and the ED
    cross-check at n=12 (GPU fDMRG against the dense ground-state energy)."""
    import torch

    import tnpy_gb300 as tg

    n, chi = 32, 32
    f = tg.FiniteDMRG(tg.model.XXZ(n, -0.5).mpo, bond_dim=chi, seed=1234, precision="fp64", compute_variance=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    es = f.run(tol=1e-8, max_sweep=10)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    out = {"workload": "fdmrg_xxz_n32_chi32_fp64", "sweeps": len(es), "seconds": dt,
           "s_per_sweep": statistics.fmean(f.sweep_seconds), "energy": es[-1], "unconverged": f.stats["unconverged"]}
    g = tg.FiniteDMRG(tg.model.XXZ(12, -0.5).mpo, bond_dim=chi, seed=1234, precision="fp64", compute_variance=False)
    e12 = g.run(tol=1e-10, max_sweep=10)[-1]
    out["n12_energy"] = e12
    if with_cpu:
        from oracle import dmrg as odmrg
        from oracle import models as om
        from oracle import operators as oops

        e_ed = float(np.linalg.eigvalsh(oops.full_hamiltonian(om.xxz_mpo(12, -0.5)))[0])
        out["ed_n12_energy"] = e_ed
        out["dE_rel_n12_vs_ed"] = abs(e12 - e_ed) / abs(e_ed)
        o = odmrg.FiniteDMRG(om.xxz_mpo(n, -0.5), chi=chi, seed=1234, eig_tol=1e-10)
        t0 = time.perf_counter()
        eo = o.run(tol=1e-8, max_sweep=10, with_variance=False)
        tc = time.perf_counter() - t0
        out["dE_rel_vs_cpu_restatement"] = abs(es[-1] - eo[-1]) / abs(eo[-1])
        out["cpu_baseline"] = {"value": len(eo) / tc, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                               "s_per_sweep": tc / len(eo), "sweeps": len(eo),
                               "sample": "the whole run (same seed, tol, sweep limit) of the numpy restatement"}
    out["value"] = len(es) / dt
    out["unit"] = "sweeps/s"
    return out


def chi_ramp_line(precision: str = "mixed"):
    """The chi ramp on XXZ(100, delta=-0.5): chi 256 -> 512 -> 1024 from the seeded random
    MPS, two sweeps per stage and then sweeps to |dE| < 1e-8 at chi=1024 (FiniteDMRG.ramp): per
    stage the sweeps, seconds, energy, middle-bond truncation error (weight beyond the previous
    chi) and smallest kept Schmidt weight, and the time to solution of the whole ramp."""
    import torch

    import tnpy_gb300 as tg

    f = tg.FiniteDMRG(tg.model.XXZ(100, -0.5).mpo, bond_dim=256, seed=1234, precision=precision,
                      compute_variance=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stages = f.ramp([256, 512, 1024], sweeps_per_stage=2, tol=1e-8, max_sweep=12)
    dt = time.perf_counter() - t0
    out = {"workload": f"fdmrg_xxz_n100_ramp256_512_1024_{precision}", "seconds_total": dt,
           "unconverged": f.stats["unconverged"], "df64_retries": f.stats["df64_retries"], "stages": []}
    for st in stages:
        out["stages"].append({k: st[k] for k in ("chi", "sweeps", "seconds", "energy", "smallest_kept_weight")
                              if k in st} | ({"truncation_error_prev_chi": st["truncation_error_prev_chi"]}
                                             if "truncation_error_prev_chi" in st else {}))
    del f
    torch.cuda.empty_cache()
    return out


def random_field_line(with_cpu: bool):
    """Random-field Heisenberg RandomHeisenberg(200, h=3, seed=7), chi=512: the mixed form with
    FP32 environment storage swept to convergence from the seeded random MPS, then the plain
    FP64 form converged from a copy of that state; seconds per sweep of each, |dE|/|E|, the
    largest difference of the middle-bond entanglement spectra and of the local <Sz_i>."""
    import torch

    import tnpy_gb300 as tg

    n, chi = 200, 512
    mpo = tg.model.RandomHeisenberg(n, h=3.0, seed=7).mpo
    f = tg.FiniteDMRG(mpo, bond_dim=chi, seed=1234, precision="mixed", env_precision="fp32", compute_variance=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # FP32-stored environments make the local eigenvalues wander by ~1e-6 between sweeps: the
    # run stops at |dE| < 1e-6 and its accuracy is read from the state (FP64 <H>, spectrum)
    em = f.run(tol=1e-6, max_sweep=10)
    torch.cuda.synchronize()
    tm = time.perf_counter() - t0
    g = tg.FiniteDMRG(mpo, bond_dim=chi, mps=tg.MatrixProductState([t.clone() for t in f.mps.tensors]),
                      precision="fp64", compute_variance=False)
    ef = g.run(tol=1e-10, max_sweep=6)
    from tnpy_gb300.matrix_product_state import expectation_value

    e_state = expectation_value(f.mps, mpo) / expectation_value(f.mps)
    bond = n // 2 - 1
    lam_m, lam_f = f.measurements.entanglement_spectrum(bond), g.measurements.entanglement_spectrum(bond)
    sz_m, sz_f = f.measurements.local_sz(), g.measurements.local_sz()
    out = {"workload": "fdmrg_random_heisenberg_n200_h3_chi512", "mixed_env": "fp32",
           "mixed": {"sweeps": len(em), "seconds": tm, "s_per_sweep_last": f.sweep_seconds[-1], "energy": em[-1],
                     "unconverged": f.stats["unconverged"], "df64_retries": f.stats["df64_retries"]},
           "fp64_from_mixed_state": {"sweeps": len(ef), "s_per_sweep_last": g.sweep_seconds[-1], "energy": ef[-1]},
           "speedup_mixed_vs_fp64_per_sweep": g.sweep_seconds[-1] / f.sweep_seconds[-1],
           "dE_rel_mixed_vs_fp64": abs(e_state - ef[-1]) / abs(ef[-1]),
           "dE_rel_mixed_local_eigenvalue_vs_fp64": abs(em[-1] - ef[-1]) / abs(ef[-1]),
           "mixed_energy_fp64_expectation": e_state,
           "spectrum_bond": bond, "spectrum_max_abs_diff": float(np.abs(lam_m - lam_f).max()),
           "spectrum_top5_fp64": lam_f[:5].tolist(), "max_sz_err_mixed_vs_fp64": float(np.abs(sz_m - sz_f).max())}
    # the same mixed run with FP64-stored environments, for the spectrum's first-order error
    h = tg.FiniteDMRG(mpo, bond_dim=chi, seed=1234, precision="mixed", compute_variance=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h.run(tol=1e-8, max_sweep=10)
    torch.cuda.synchronize()
    lam_h = h.measurements.entanglement_spectrum(bond)
    e_h = expectation_value(h.mps, mpo) / expectation_value(h.mps)
    out["mixed_fp64_env"] = {"sweeps": len(h.sweep_seconds), "seconds": time.perf_counter() - t0,
                             "s_per_sweep_last": h.sweep_seconds[-1],
                             "dE_rel_vs_fp64": abs(e_h - ef[-1]) / abs(ef[-1]),
                             "spectrum_max_abs_diff_vs_fp64": float(np.abs(lam_h - lam_f).max())}
    del f, g, h
    torch.cuda.empty_cache()
    return out


def tsdrg_rate(n_real: int, with_cpu: bool, n_single: int = 16):
    """Batched tSDRG on `n_real` random-coupling chains J_i = (1-u_i)^(1/delta), u = RandomState(10000+r),
    n=128, chi=32, delta=1, h=0 (realisations/s): all realisations merged in lockstep (one launch
    of each kernel per merge step for every chain), FP64 and mixed; against one realisation per
    launch sequence (TSDRG(mpo, chi).run() one after another, FP64) on the first `n_single`
    realisations, with their kept spectra compared; and the CPU restatement (one realisation)
    timed on the host cores beside it. The h=0 chain is SU(2) symmetric, so the comparison with
    the CPU restatement's kept spectra is made on the h=0.5 variant (two realisations)."""
    import torch

    import tnpy_gb300 as tg

    n, chi = 128, 32
    mpos = [tg.model.RandomCouplingHeisenberg(n, delta=1.0, seed=10000 + r).mpo for r in range(n_real)]
    tg.BatchedTSDRG(mpos[:2], chi=chi).run()  # warm-up (kernels, workspaces)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = tg.BatchedTSDRG(mpos, chi=chi).run()  # FP64 (the reference's arithmetic)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    t0 = time.perf_counter()
    bm = tg.BatchedTSDRG(mpos, chi=chi, precision="mixed").run()
    torch.cuda.synchronize()
    dtm = time.perf_counter() - t0
    ns = min(n_single, n_real)
    t0 = time.perf_counter()
    singles = []
    for r in range(ns):
        t = tg.TSDRG(mpos[r], chi=chi)
        t.run()
        singles.append(t.evals)
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    diff = max(float(np.abs(np.asarray(singles[r]) - np.asarray(b.evals[r])).max()) for r in range(ns))
    single_rate = ns / ts
    out = {"workload": f"tsdrg_random_coupling_n{n}_chi{chi}_delta1_h0", "realizations": n_real,
           "value": n_real / dt, "unit": "realizations/s", "precision": "fp64", "seconds": dt,
           "mixed": {"value": n_real / dtm, "seconds": dtm, "e0_realization0": float(bm.evals[0][0])},
           "one_per_launch_fp64": {"value": single_rate, "realizations": ns, "seconds": ts,
                                   "max_abs_diff_kept_spectra_vs_batched": diff},
           "speedup_batched_vs_one_per_launch": (n_real / dt) / single_rate,
           "speedup_batched_mixed_vs_one_per_launch": (n_real / dtm) / single_rate,
           "e0_realization0": float(b.evals[0][0]),
           "note": "h=0 is SU(2) symmetric: chi=32 cuts through degenerate multiplets, so the kept states "
                   "(and the variational energy) depend on rounding in any implementation"}
    if with_cpu:
        from oracle import models as om
        from oracle import tsdrg as ots

        m = tg.model.RandomCouplingHeisenberg(n, delta=1.0, seed=10000)
        t0 = time.perf_counter()
        ots.TreeTensorNetworkSDRG(om.random_coupling_heisenberg_mpo(n, m.couplings, 0.0), chi).run()
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / tc, "unit": "realizations/s", "cores": os.cpu_count(),
                               "kind": "port", "sample": "one realisation (r=0) of the numpy restatement"}
        # kept spectra against the one-block-at-a-time FP64 numpy eigh on the h != 0 variant
        diffs, same = [], True
        mh = [tg.model.RandomCouplingHeisenberg(n, delta=1.0, h=0.5, seed=10000 + r) for r in range(2)]
        bh = tg.BatchedTSDRG([x.mpo for x in mh], chi=chi).run()
        for r, x in enumerate(mh):
            o = ots.TreeTensorNetworkSDRG(om.random_coupling_heisenberg_mpo(n, x.couplings, fields=x.fields), chi).run()
            diffs.append(float(np.abs(np.asarray(bh.evals[r]) - o.evals).max()))
            same = same and [list(q) for q in bh.merges[r]] == [list(q) for q in o.merges]
        out["parity_h05_vs_cpu_restatement"] = {"realizations": 2, "max_abs_diff_kept_spectra": max(diffs),
                                                "merge_order_equal": same}
    return out


def chains_rate(n_chains: int, with_cpu: bool, n_single: int = 4, precision: str = "mixed"):
    """Many independent chains: RandomHeisenberg(64, h=1, seed=100+c) at chi=64 swept in lockstep
    (BatchedFiniteDMRG: every kernel spans all chains, per-chain Davidson convergence masks) to
    |dE| < 1e-8 per chain (at most 10 sweeps), in the batched mixed form (double-FP32 products
    on the FP32 pipe, FP64 Rayleigh-Ritz); against one chain per launch sequence (FiniteDMRG per
    chain, one after another) on the first `n_single` chains, whose final energies are compared;
    and one sweep of one chain of the CPU restatement."""
    import torch

    import tnpy_gb300 as tg

    n, chi = 64, 64
    mpos = [tg.model.RandomHeisenberg(n, h=1.0, seed=100 + c).mpo for c in range(n_chains)]
    tg.BatchedFiniteDMRG(mpos[:2], bond_dim=chi, seed=100, precision=precision).run(tol=1e-8, max_sweep=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = tg.BatchedFiniteDMRG(mpos, bond_dim=chi, seed=100, precision=precision)
    eb = b.run(tol=1e-8, max_sweep=10)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    sweeps = sum(b.sweeps)
    ns = min(n_single, n_chains)
    t0 = time.perf_counter()
    singles = []
    for c in range(ns):
        f = tg.FiniteDMRG(mpos[c], bond_dim=chi, seed=100 + c, precision="fp64", compute_variance=False)
        singles.append(f.run(tol=1e-8, max_sweep=10)[-1])
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    de = max(abs(eb[c][-1] - singles[c]) / abs(singles[c]) for c in range(ns))
    out = {"workload": f"fdmrg_random_heisenberg_n{n}_chi{chi}_h1_chains{n_chains}", "chains": n_chains,
           "engine": "BatchedFiniteDMRG (lockstep, every kernel spans all chains)", "precision": precision,
           "value": n_chains / dt, "unit": "chains/s", "chain_sweeps_per_s": sweeps / dt, "sweeps_total": sweeps,
           "lockstep_sweeps": len(b.sweep_seconds), "seconds": dt, "e0_chain0": float(eb[0][-1]),
           "unconverged_local_solves": b.stats["unconverged"],
           "one_chain_per_launch_fp64": {"value": ns / ts, "unit": "chains/s", "chains": ns, "seconds": ts},
           "speedup_vs_one_chain_per_launch": (n_chains / dt) / (ns / ts),
           "max_dE_rel_vs_one_chain_per_launch": de}
    del b
    torch.cuda.empty_cache()
    if with_cpu:
        from oracle import dmrg as odmrg
        from oracle import models as om

        o = odmrg.FiniteDMRG(om.random_heisenberg_mpo(n, 1.0, seed=100), chi=chi)
        t0 = time.perf_counter()
        o.sweep(True, 1e-8)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / tc, "unit": "chain-sweeps/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "first (rightward) sweep of chain 0 of the numpy restatement"}
    return out


# ------------------------------------------------------------------ reference arm
def run_reference(a):
    """The reference's CPU path (numpy/scipy restatement; quimb and primme cannot be installed
    here) on the bench's chain: one step = one real site update of a sweep (see CpuBulkPair),
    on the machine's host cores with every thread BLAS can use. Untimed set-up builds the seeded
    random MPS of the GPU arm and converges the bulk pair; then W warm-up and K timed updates."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    t_setup = time.perf_counter()
    pair = CpuBulkPair(*cpu_pair_from_random_mps(a), tol=a.tol)
    setup_s = time.perf_counter() - t_setup
    res = cpu_site_updates(pair, a.steps, a.warmup, prepare_s=120.0)
    cb = cpu_result(a, res, "state: a seeded random MPS whose middle pair has the bench chain's bulk local "
                            "problem shape (chi x D x chi environments), converged before the warm-up")
    cb["setup_s"] = setup_s
    ms = statistics.fmean(res["times"]) * 1e3
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "sweeps/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random MPS, XXZ MPO)",
            "config": workload(a), "cpu_baseline": cb,
            "step_note": "a step is one site update of the sweep (ms_per_step); value = 1 / (mean site update "
                         "x sweep_site_weight) sweeps/s",
            "e2e": {"value": cb["value"], "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ our arm
def max_over_ranks(x: float, device) -> float:
    """Largest x over the ranks of the default process group (x itself without one): the
    whole-job step time is that of the slowest replica."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(a):
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import tnpy_gb300 as tg
    from tnpy_gb300._lib import lib
    import ctypes

    dev = torch.device("cuda", local)
    mpo = tg.model.XXZ(a.n, a.delta).mpo
    f = tg.FiniteDMRG(mpo, bond_dim=a.chi, precision=a.precision, seed=a.seed + rank, compute_variance=False,
                      device=dev)
    dirs = [tg.Direction.RIGHTWARD, tg.Direction.LEFTWARD]
    step = 0
    energies = []

    def one_sweep():
        nonlocal step
        e = f.sweep(dirs[step % 2], tol=a.tol)
        step += 1
        energies.append(e)
        return e

    # warm-up sweeps from the random MPS (the convergence the timed, converged sweeps follow):
    # host wall time of each (device synchronised) and its energy
    warmup_s = []
    for _ in range(a.warmup):
        torch.cuda.synchronize()
        tw = time.perf_counter()
        one_sweep()
        torch.cuda.synchronize()
        warmup_s.append(time.perf_counter() - tw)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timed region
    clocks = Clocks(local)
    barrier()
    launches0 = lib.tnx_launch_count()  # library launches before the timed region (ncu -s windows)
    lib.tnx_profile_begin(6)  # Ozaki FP64-class GEMM: the headline roofline's kernel
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mv0, it0 = f.stats["matvecs"], f.stats["iterative_solves"]
    ev0.record()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        one_sweep()
    ev1.record()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    mv_timed = (f.stats["matvecs"] - mv0) / max(1, f.stats["iterative_solves"] - it0)
    launches = lib.tnx_launch_count() - launches0
    n_o, ms_o, fl_o, by_o = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
    lib.tnx_profile_end(ctypes.byref(n_o), ctypes.byref(ms_o), ctypes.byref(fl_o), ctypes.byref(by_o))
    dev_ms = ev0.elapsed_time(ev1)
    t_step = max_over_ranks(dev_ms / 1e3 / a.steps, dev)
    value = world / t_step

    # ---- end-to-end: MPS round-trips through pinned host memory every step
    host = [torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in f.mps.tensors]
    for h, t in zip(host, f.mps.tensors):
        h.copy_(t)
    h2d = sum(h.numel() * 8 for h in host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        for h, t in zip(host, f.mps.tensors):
            t.copy_(h, non_blocking=True)
        e = one_sweep()
        for h, t in zip(host, f.mps.tensors):
            h.copy_(t, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    barrier()
    e2e_t = max_over_ranks((time.perf_counter() - t0) / a.steps, dev)

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_sust = peaks.get("bf16_tflops_sustained")
    peak_src = "of measured"
    if bf16_sust is None:
        bf16_sust, peak_src = 1700.0, "of fallback (1.7 PFLOP/s sustained bf16)"
    tf = ROOT / "profiles" / "traffic.txt"

    def traffic_of(key):
        if tf.exists():
            for ln in tf.read_text().splitlines():
                parts = ln.split()
                if len(parts) == 2 and not ln.startswith("#") and parts[0] == key:
                    return float(parts[1])
        return None

    # Every kernel family of the step: the Ozaki GEMM over the timed sweeps (CUDA events around
    # each launch, library profiler); the others over one further sweep each, outside the timed
    # region. The headline roofline is the family with the largest share of the step.
    fams = {0: ("bf16x3_gemm_kernel (tcgen05 split-BF16 GEMM of the one-site matvec)", 3.0,
                "bf16_tflops_sustained / 3 (three BF16 products per split-BF16 product)", f"tc_gemm_chi{a.chi}"),
            1: ("gemm_df64_kernel + nar_* (double-FP32 / FP64 SIMT GEMMs: the QR's next-panel update and "
                "small T products, products too small for the tensor-core GEMM)", 36.0,
                "bf16_tflops_sustained / 36, the FP64-class tensor-core bound the Ozaki GEMM runs against "
                "(this SIMT kernel does the same FP64-class products on the FP32 pipe)", None),
            3: ("qrdf::panel_df_kernel (double-FP32 16-CTA cluster Householder panel)", 36.0,
                "bf16_tflops_sustained / 36 (FP64-class tensor-core bound)", None),
            6: ("oz_gemm_kernel (tcgen05 FP64-class GEMM, 36 exact BF16 slice products: environment updates, "
                "anchor matvecs, the gauge move's X, Q and R A)", 36.0,
                "bf16_tflops_sustained / 36 (36 BF16 slice products per FP64-class product)", f"oz_gemm_chi{a.chi}"),
            7: ("oz_gemm_kernel[narrow] (the same kernel on the QR's K = 64 and split-K trailing / WY products)",
                36.0, "bf16_tflops_sustained / 36 (36 BF16 slice products per FP64-class product)", None)}
    prof = {6: (n_o.value, ms_o.value, fl_o.value, dev_ms, a.steps)}
    for fam in (0, 1, 3, 7):
        lib.tnx_profile_begin(fam)
        sw0, sw1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sw0.record()
        one_sweep()
        sw1.record()
        n_f, ms_f, fl_f, by_f = ctypes.c_int(0), ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
        lib.tnx_profile_end(ctypes.byref(n_f), ctypes.byref(ms_f), ctypes.byref(fl_f), ctypes.byref(by_f))
        torch.cuda.synchronize()
        prof[fam] = (n_f.value, ms_f.value, fl_f.value, sw0.elapsed_time(sw1), 1)

    def roofline_of(fam):
        n_l, ms_l, fl_l, sweep_ms, sweeps = prof[fam]
        name, div, note, tkey = fams[fam]
        ach = fl_l / (ms_l / 1e3) / 1e12 if ms_l > 0 and fl_l > 0 else None
        pk = bf16_sust / div
        return {"kernel": name, "bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                "frac": (ach / pk) if ach else None, "traffic": traffic_of(tkey) if tkey else None,
                "launches": n_l, "kernel_ms_per_sweep": ms_l / sweeps,
                "share_of_step_time": (ms_l / sweep_ms) if sweep_ms > 0 else None,
                "peak_note": f"{peak_src}: {note}; achieved = algorithmic flops (2 M N K per GEMM, "
                             f"3 m nb^2 per QR panel) / summed CUDA-event time of the family's launches",
                "window": "the timed sweeps" if fam == 6 else "one profiled sweep after the timed ones"}

    rooflines = {fam: roofline_of(fam) for fam in prof}
    shares = {fams[f][0].split(" ")[0]: {"launches": r["launches"], "ms_per_sweep": r["kernel_ms_per_sweep"],
                                         "share": r["share_of_step_time"], "tflops": r["achieved"]}
              for f, r in rooflines.items()}
    top = max(rooflines, key=lambda f: rooflines[f]["share_of_step_time"] or 0.0)
    # the timed-sweep counters of the Davidson: unconverged solves are retried in FP64 and warned
    dstats = dict(f.stats)

    # time to solution from the seeded random MPS: warm-up sweeps until |dE| < tol
    conv_at, acc = None, 0.0
    for k_s, (ts, es) in enumerate(zip(warmup_s, energies)):
        acc += ts
        if k_s > 0 and abs(es - energies[k_s - 1]) < a.tol:
            conv_at = {"sweeps": k_s + 1, "s": acc, "energy": es}
            break

    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (split-bf16 tensor-core matvec, FP64-class environments / gauge "
            "moves, FP64 eigensolver)" if a.precision == "mixed" else "f64",
            "data": "synthetic (seeded random initial MPS, XXZ MPO)", "config": workload(a),
            "roofline": rooflines[top], "roofline_ozaki": rooflines[6], "roofline_ozaki_narrow": rooflines[7],
            "roofline_matvec": rooflines[0],
            "step_shares": shares, "clocks": clk, "gpu_launches": int(launches),
            "e2e": {"value": world / e2e_t, "unit": "sweeps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": h2d + 8},
            "energy_last": energies[-1], "wall_s_per_step": wall / a.steps,
            "davidson_matvecs_per_site_timed": mv_timed, "launches_before_timed": int(launches0),
            "davidson": {"unconverged": dstats["unconverged"], "df64_retries": dstats["df64_retries"],
                         "iterative_solves": dstats["iterative_solves"], "matvecs": dstats["matvecs"],
                         "window": "warm-up, timed, e2e and profiled sweeps"},
            "warmup_sweeps": {"s": warmup_s, "energy": energies[:a.warmup]},
            "first_sweep_s": warmup_s[0] if warmup_s else None,
            "time_to_convergence": conv_at}
    if rank == 0 and not a.no_extras:
        line["matvec_forms"] = matvec_forms(f, a.n // 2)
        line["fp64_sweep"] = fp64_sweep(f, dirs[step % 2], a.tol, t_step)
        line["xxz_n32_chi32_fp64"] = xxz_n32_line(with_cpu=(world == 1 and not a.no_cpu))
        line["xxz_n100_chi_ramp"] = chi_ramp_line()
        line["random_heisenberg_n200_chi512"] = random_field_line(with_cpu=(world == 1 and not a.no_cpu))
        line["tsdrg"] = tsdrg_rate(a.tsdrg_realizations, with_cpu=(world == 1 and not a.no_cpu))
        line["chains"] = chains_rate(a.chains, with_cpu=(world == 1 and not a.no_cpu))
    if rank == 0 and world == 1 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline_converged(f, a, dirs[step % 2])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline_converged(f, a, direction):
    """CPU restatement timed on the GPU chain's own converged state: the GPU chain sweeps (in
    `direction`) up to its middle site, the bulk pair there (L_i, R_{i+1}, the two site tensors,
    their MPO tensors) is copied to the host, the sweep is completed on the GPU, and the CPU
    restatement performs 2 warm-up and 8 timed site updates on the copy (about 10-20 s)."""
    import numpy as np

    import tnpy_gb300 as tg

    n = f.n_sites
    i = n // 2
    sites = list(range(n - 1)) if direction == tg.Direction.RIGHTWARD else list(range(n - 1, 0, -1))

    def update(site):
        e, psi = f.one_site_solver(site, a.tol)
        f.env.update_mps(site, psi)
        f.perturb_wave_function(site)
        f.env.split_tensor(site, direction)
        f.env.update(site, direction)

    k = sites.index(i)
    for site in sites[:k]:
        update(site)
    w = f.env.mpo.device_tensors(f.mps.device)
    host = lambda t: t.detach().cpu().numpy().astype(np.float64)  # noqa: E731
    data = (host(f.env.left[i]), host(w[i]), host(w[i + 1]), host(f.env.right[i + 1]),
            host(f.mps.tensors[i]), host(f.mps.tensors[i + 1]))
    for site in sites[k:]:
        update(site)
    pair = CpuBulkPair(*data, tol=a.tol)
    res = cpu_site_updates(pair, steps=8, warmup=2)
    return cpu_result(a, res, "state: the GPU chain's converged bulk pair after the timed sweeps")


def main():
    a = parse()
    if a.impl == "reference":
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
