"""One-site finite DMRG on the GPU (tnpy/finite_dmrg.py:22-263).

Drop-in for ``FiniteDMRG(mpo, bond_dim).run(tol)`` and the README spelling
``FiniteDMRG(mpo=..., chi=...).update(tol=...)``. Per site the sweep keeps the
reference's steps (:143-171): lowest eigenpair of the one-site effective
Hamiltonian (dense Jacobi below ``exact_solver_dim`` elements, device Davidson
above), the 1e-5 perturbation psi += 1e-5 H_eff psi (:116-141), the gauge move
onto the neighbour (QR form), and the environment update.

``precision='mixed'`` runs the Davidson matvecs as split-BF16 tensor-core
contractions and certifies each local eigenpair with FP64-class anchor matvecs
(Ozaki-sliced FP64 GEMMs on the tensor cores), runs environment updates in the
same FP64-class form and gauge moves with double-FP32 QR panels and updates;
Rayleigh-Ritz stays FP64.
"""
from __future__ import annotations

import logging
import time
from concurrent.futures import ThreadPoolExecutor
from enum import Enum
from itertools import cycle

import numpy as np
import torch

from . import kernels as K
from .matrix_product_state import (
    Direction,
    Environment,
    MatrixProductState,
    MatrixProductStateMeasurements,
)
from .operators import MatrixProductOperator

logger = logging.getLogger("tnpy")


class Metric(Enum):
    """tnpy/finite_dmrg.py:22-29."""

    ENERGY = 1
    VARIANCE = 2


class FiniteDMRG:
    def __init__(
        self,
        mpo: MatrixProductOperator,
        bond_dim: int | None = None,
        block_size: int = 1,
        mps: MatrixProductState | None = None,
        exact_solver_dim: int = 200,
        *,
        chi: int | None = None,
        precision: str = "fp64",
        seed: int | None = 1234,
        max_iter: int = 400,
        max_basis: int = 24,
        compute_variance: bool = True,
        device=None,
        env_precision: str = "fp64",
    ):
        if bond_dim is None:
            bond_dim = chi
        if bond_dim is None:
            raise TypeError("FiniteDMRG needs bond_dim (or chi)")
        if block_size != 1:
            raise NotImplementedError("only the one-site update (block_size=1) is on this path")
        self._n_sites = mpo.n_sites
        self._bond_dim = int(bond_dim)
        self._phys_dim = mpo.phys_dim
        self._block_size = block_size
        self._exact_solver_dim = exact_solver_dim
        self.precision = precision
        K.precision_code(precision)
        self.max_iter = max_iter
        self.max_basis = max_basis
        self.compute_variance = compute_variance
        if mps is None:
            mps = MatrixProductState.random(self._n_sites, self._bond_dim, self._phys_dim, seed=seed, device=device)
        env_dtypes = {"fp64": torch.float64, "fp32": torch.float32}
        if env_precision not in env_dtypes:
            raise ValueError(f"env_precision must be 'fp64' or 'fp32', not {env_precision!r}")
        self._env = Environment(mpo=mpo, mps=mps, precision=precision, env_dtype=env_dtypes[env_precision])
        self._energies = [np.nan]
        self._variances = [np.nan]
        self.sweep_seconds: list[float] = []
        self.stats = {"matvecs": 0, "dense_solves": 0, "iterative_solves": 0, "unconverged": 0,
                      "df64_retries": 0}
        # sites whose last mixed solve converged at its first anchor, with no split-BF16 expansion
        self._settled: dict[int, bool] = {}

    # ---- properties (finite_dmrg.py:78-95) ----------------------------------------------
    @property
    def bond_dim(self) -> int:
        return self._bond_dim

    chi = bond_dim

    @property
    def mps(self) -> MatrixProductState:
        return self._env.mps

    @property
    def env(self) -> Environment:
        return self._env

    @property
    def n_sites(self) -> int:
        return self._n_sites

    @property
    def phys_dim(self) -> int:
        return self._phys_dim

    @property
    def energies(self) -> list[float]:
        return self._energies[1:]

    def variance(self) -> float:
        return self._env.variance()

    # ---- local steps --------------------------------------------------------------------
    def one_site_solver(self, site: int, tol: float = 1e-8, **kwargs):
        """Lowest eigenpair at ``site`` (finite_dmrg.py:97-111). Returns (energy, psi) with
        psi a device tensor of the site's shape.

        An iterative solve that ends without meeting ``tol`` is never passed on silently (the
        reference's primme.eigsh raises on non-convergence by default): a mixed-precision
        solve is first continued by the FP64-class Davidson ('df64': Ozaki-sliced FP64 products
        on the tensor cores) from the vector it reached (``stats['df64_retries']``); a solve
        that still fails is logged as a warning on the
        ``tnpy`` logger and counted in ``stats['unconverged']``, or raises RuntimeError with
        ``raise_on_fail=True``."""
        x = self.mps.tensors[site]
        if x.numel() < self._exact_solver_dim:
            self.stats["dense_solves"] += 1
            h = self._env.one_site_full_matrix(site)
            evals, evecs = K.eigh_batched([h], keep=1)
            return float(evals[0, 0].item()), evecs[0, :, 0].reshape(x.shape).contiguous()
        self.stats["iterative_solves"] += 1
        psi = x.clone()
        L, W, R = self._env.site_operator(site)
        max_iter = kwargs.get("max_iter", self.max_iter)
        max_basis = kwargs.get("max_basis", self.max_basis)
        precision = kwargs.get("precision", self.precision)
        # a site whose last solve needed nothing beyond the anchor's certification starts there
        mixed = K.precision_code(precision) == K.precision_code("mixed")
        start_anchored = mixed and self._settled.get(site, False)
        e, rn, its, ok = K.davidson1(L, W, R, psi, tol=tol, max_iter=max_iter, max_basis=max_basis,
                                     precision=precision, start_anchored=start_anchored)
        if mixed:
            st = K.davidson1_stats()
            self._settled[site] = bool(ok and st["anchored"] == 0 and st["anchors"] == 1 and st["phase1"] <= 1)
            self.stats["anchored_starts"] = self.stats.get("anchored_starts", 0) + int(start_anchored)
        self.stats["matvecs"] += its
        if not ok and K.precision_code(precision) == K.precision_code("mixed"):
            self.stats["df64_retries"] += 1
            logger.info(f"site {site}: {precision} Davidson stopped at residual {rn:.3e} after {its} matvecs; "
                        f"continuing in FP64-class arithmetic")
            e, rn, its, ok = K.davidson1(L, W, R, psi, tol=tol, max_iter=max_iter, max_basis=max_basis,
                                         precision="df64")
            self.stats["matvecs"] += its
        if not ok:
            self.stats["unconverged"] += 1
            msg = f"site {site}: Davidson did not converge (residual {rn:.3e} after {its} matvecs, tol {tol:.1e})"
            if kwargs.get("raise_on_fail", False):
                raise RuntimeError(msg)
            logger.warning(msg)
        return e, psi

    def two_site_solver(self, site: int, tol: float = 1e-8, **kwargs):
        return NotImplemented

    def enlarge_bond_dim(self, new_bond_dim: int, seed: int | None = 0):
        """Grow the bond dimension to ``new_bond_dim`` (MatrixProductState.enlarge_bond_dim) and
        rebuild the environments; call with the centre on site 0, i.e. before a rightward
        sweep. One-site sweeps then fill the new directions (bond-dimension ramp)."""
        self.mps.enlarge_bond_dim(new_bond_dim, seed=seed)
        self._bond_dim = int(new_bond_dim)
        self._env.rebuild()
        self._settled.clear()

    def ramp(self, bond_dims, sweeps_per_stage: int = 2, tol: float = 1e-8, max_sweep: int = 20,
             bond: int | None = None, **kwargs) -> list[dict]:
        """Bond-dimension ramp (a builder addition: the reference fixes the bond dimension of its
        one-site DMRG, finite_dmrg.py:113-114 and matrix_product_state.py:227-228 are stubs).

        For each chi in ``bond_dims`` the MPS is grown to chi (``enlarge_bond_dim``, the state
        unchanged) and swept: ``sweeps_per_stage`` sweeps (rounded up to an even number, so that
        a stage ends leftward with the centre on site 0, where the next enlargement needs it),
        and on the last stage until |dE| < tol after a leftward sweep or ``max_sweep`` sweeps.
        After each stage the Schmidt values on ``bond`` (default: the middle bond) are computed
        by a direct FP64 SVD. The truncation error of stage k is the weight its state would
        lose at that bond if cut back to the previous stage's chi, sum_{j > chi_(k-1)} lambda_j^2:
        the discarded weight a chi_(k-1) calculation commits there, as measured by the larger
        state (the last stage reports the smallest kept weight lambda_chi^2 beside it).
        Returns one dict per stage: chi, sweeps, energy, seconds, spectrum (host array),
        truncation_error_prev_chi and smallest_kept_weight."""
        bond = self.n_sites // 2 - 1 if bond is None else int(bond)
        stages: list[dict] = []
        per = sweeps_per_stage + (sweeps_per_stage % 2)
        for k, chi in enumerate(bond_dims):
            if chi != self.bond_dim:
                self.enlarge_bond_dim(int(chi))
            last = k == len(bond_dims) - 1
            n_sw = max_sweep if last else per
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            es: list[float] = []
            for j in range(n_sw):
                direction = Direction.RIGHTWARD if j % 2 == 0 else Direction.LEFTWARD
                e = self.sweep(direction, tol=tol, **kwargs)
                es.append(e)
                self._energies.append(e)
                self._variances.append(np.nan)
                if last and j % 2 == 1 and len(es) >= 2 and abs(es[-1] - es[-2]) < tol:
                    break
            torch.cuda.synchronize()
            lam = MatrixProductStateMeasurements(self.mps).entanglement_spectrum(bond)
            stage = {"chi": int(chi), "sweeps": len(es), "energy": es[-1], "energies": es,
                     "seconds": time.perf_counter() - t0, "spectrum": lam,
                     "smallest_kept_weight": float(lam[-1] ** 2)}
            if stages:
                prev = stages[-1]["chi"]
                stage["truncation_error_prev_chi"] = float(np.sum(lam[prev:] ** 2))
            stages.append(stage)
        return stages

    def perturb_wave_function(self, site: int, alpha: float = 1e-5):
        """psi += alpha H_eff psi, in place, not renormalised (finite_dmrg.py:116-141)."""
        psi = self.mps.tensors[site]
        L, W, R = self._env.site_operator(site)
        hpsi = K.matvec1(L, W, R, psi, precision=self.precision)
        psi.add_(hpsi, alpha=alpha)

    def sweep(self, direction: Direction = Direction.RIGHTWARD, tol: float = 1e-8, **kwargs) -> float | None:
        """One sweep (finite_dmrg.py:143-171)."""
        sites = range(self.n_sites - 1) if direction == Direction.RIGHTWARD else range(self.n_sites - 1, 0, -1)
        energy = None
        for site in sites:
            energy, psi = self.one_site_solver(site, tol, **kwargs)
            logger.debug(f"Sweeping to site [{site + 1}/{self.n_sites}], E0 = {energy}")
            self._env.update_mps(site, psi)
            self.perturb_wave_function(site)
            self._env.split_tensor(site, direction=direction)
            self._env.update(site, direction=direction)
        return energy

    def _converged(self, n_sweep: int, tol: float, max_sweep: int, metric: Metric) -> bool:
        """finite_dmrg.py:173-212."""
        values = self._variances if metric == Metric.VARIANCE else self._energies
        gradient = float(np.diff(values[-2:])[0])
        logger.info(f"Metric {metric.name} is lowered by {gradient:e} in this sweep.")
        if abs(gradient) < tol:
            logger.info(f"Reaching set tolerance {tol}, stop sweeping.")
            return True
        if n_sweep == max_sweep:
            logger.warning(f"Maximum number of sweeps {max_sweep} is reached, yet {metric.name} "
                           f"gradient = {gradient:e} is still greater than tol = {tol}.")
        elif abs(gradient) > tol and gradient < 0:
            logger.warning(f"Might be trapped in local minimum in this sweep, got {metric.name} "
                           f"gradient = {gradient:e}, skip and proceed.")
        return False

    def run(self, tol: float = 1e-8, max_sweep: int = 100, metric: Metric = Metric.ENERGY, **kwargs) -> list[float]:
        """Sweep until |dE| < tol or ``max_sweep`` (finite_dmrg.py:214-257). Returns the
        energy of every sweep. Sweep wall times (device-synchronised) go to
        ``sweep_seconds``; the variance is not part of the timed sweep, as in the reference."""
        logger.info(f"Set tolerance = {tol} to metric {metric.name}, up to maximally {max_sweep} sweeps.")
        n_sweep = 0
        for n_sweep, direction in zip(range(1, max_sweep + 1), cycle([Direction.RIGHTWARD, Direction.LEFTWARD])):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            energy = self.sweep(direction, tol=tol, **kwargs)
            torch.cuda.synchronize()
            self.sweep_seconds.append(time.perf_counter() - t0)
            self._energies.append(energy)
            if self.compute_variance or metric == Metric.VARIANCE:
                self._variances.append(self._env.variance())
            else:
                self._variances.append(np.nan)
            if self._converged(n_sweep, tol, max_sweep, metric):
                break
        best = np.mean(np.sort(self.sweep_seconds)[:3]) if self.sweep_seconds else 0.0
        logger.info(f"Summary - {n_sweep} sweeps, best of {min(3, n_sweep)} - {best:.6f} s per sweep.")
        return self._energies[1:]

    update = run

    @property
    def measurements(self) -> MatrixProductStateMeasurements:
        if len(self._energies) == 1:
            raise RuntimeError("FiniteDMRG is probably not executed yet.")
        return MatrixProductStateMeasurements(self.mps)


class ShiftInvertDMRG(FiniteDMRG):
    """Shift-invert one-site DMRG for excited states near an energy eps (tnpy/finite_dmrg.py:266-407).

    ``mpo`` is the MPO of H - eps (e.g. RandomHeisenberg(..., offset=eps)); every site solves the
    generalised problem (H - eps) phi = lambda (H - eps)^2 phi for the smallest lambda, with the
    second operator from environments of the MPO square (bond D^2): densely below
    ``exact_solver_dim`` elements (B^-1/2 A B^-1/2 from the device Jacobi eigensolver), else by
    the device generalised Davidson (tnx_gdavidson1, B-orthonormal basis). ``run`` returns the
    energies 1/lambda + offset of every sweep and restores psi = (H - eps) phi site by site
    (tnx_mpo_apply_site); ``measurements`` and ``variance`` act on the restored state."""

    def __init__(self, mpo: MatrixProductOperator, bond_dim: int | None = None, offset: float = 0.0,
                 block_size: int = 1, mps: MatrixProductState | None = None, exact_solver_dim: int = 200, *,
                 chi: int | None = None, precision: str = "fp64", seed: int | None = 1234, max_iter: int = 400,
                 max_basis: int = 48, device=None):
        if precision == "mixed":
            raise ValueError("shift-invert DMRG runs in 'fp64' or the FP64-class 'df64' form")
        super().__init__(mpo, bond_dim, block_size, mps, exact_solver_dim, chi=chi, precision=precision, seed=seed,
                         max_iter=max_iter, max_basis=max_basis, compute_variance=False, device=device)
        self._env2 = Environment(mpo=mpo.square(), mps=self.mps, precision=precision)
        self._offset = float(offset)
        self._restored_mps: MatrixProductState | None = None

    @property
    def offset(self) -> float:
        return self._offset

    @property
    def restored_mps(self) -> MatrixProductState | None:
        return self._restored_mps

    def _restore_mps(self):
        """psi = (H - eps) phi: each site tensor contracted with its MPO tensor (:314-343)."""
        ws = self._env.mpo.device_tensors(self.mps.device)
        self._restored_mps = MatrixProductState([K.mpo_apply_site(a, w) for a, w in zip(self.mps.tensors, ws)],
                                                device=self.mps.device)

    def one_site_solver(self, site: int, tol: float = 1e-8, **kwargs):
        """Smallest generalised eigenpair at ``site`` (:345-363); the vector is B-normalised."""
        x = self.mps.tensors[site]
        if x.numel() < self._exact_solver_dim:
            self.stats["dense_solves"] += 1
            return self._dense_solve(site, x)
        self.stats["iterative_solves"] += 1
        psi = x.clone()
        L, W, R = self._env.site_operator(site)
        L2, W2, R2 = self._env2.site_operator(site)
        e, rn, its, ok = K.gdavidson1(L, W, R, L2, W2, R2, psi, tol=tol,
                                      max_iter=kwargs.get("max_iter", self.max_iter),
                                      max_basis=kwargs.get("max_basis", self.max_basis), precision=self.precision)
        self.stats["matvecs"] += its
        if not ok:
            if x.numel() <= self.DENSE_FALLBACK_DIM:
                # pencils with an ill-conditioned B can stall the Davidson far from its target:
                # solve such a site densely instead
                self.stats["dense_fallbacks"] = self.stats.get("dense_fallbacks", 0) + 1
                logger.info(f"site {site}: generalised Davidson stalled (residual {rn:.3e}); dense solve")
                return self._dense_solve(site, x)
            self.stats["unconverged"] += 1
            logger.warning(f"site {site}: generalised Davidson did not converge (residual {rn:.3e}, {its} expansions)")
        return e, psi

    DENSE_FALLBACK_DIM = 4096

    def _dense_solve(self, site: int, x: torch.Tensor):
        """Smallest eigenpair of the dense pencil: B^-1/2 A B^-1/2 (B^-1/2 from the eigenpairs of
        B) and its lowest eigenvector mapped back, as scipy.linalg.eigh(a, b) does by Cholesky."""
        from .exact_diagonalization import eigh_full

        a = self._env.one_site_full_matrix(site)
        b = self._env2.one_site_full_matrix(site)
        n = a.shape[0]
        sym = lambda m: (0.5 * (m + m.T)).contiguous()
        if n < 200:
            wb, ub = K.eigh_batched([sym(b)], keep=n)
            wb, ub = wb[0], ub[0, :n, :]
        else:
            wbh, ub = eigh_full(sym(b))
            wb = torch.as_tensor(wbh.copy(), device=b.device)
        if float(wb.min().item()) <= 0.0:
            raise RuntimeError(f"site {site}: the squared operator is not positive definite")
        bih = K.gemm((ub * wb.rsqrt()[None, :]).contiguous(), ub, trans_b=True)  # B^-1/2
        c = K.gemm(bih, K.gemm(a, bih))
        if n < 200:
            wc, uc = K.eigh_batched([sym(c)], keep=1)
            lam, u0 = float(wc[0, 0].item()), uc[0, :n, :1]
        else:
            wch, uc = eigh_full(sym(c))
            lam, u0 = float(wch[0]), uc[:, :1]
        vec = K.gemm(bih, u0.contiguous())
        return lam, vec.reshape(x.shape).contiguous()

    def sweep(self, direction: Direction = Direction.RIGHTWARD, tol: float = 1e-8, **kwargs) -> float | None:
        """:365-384: the FiniteDMRG site update, plus the MPO-square environments."""
        sites = range(self.n_sites - 1) if direction == Direction.RIGHTWARD else range(self.n_sites - 1, 0, -1)
        energy = None
        for site in sites:
            energy, psi = self.one_site_solver(site, tol, **kwargs)
            logger.debug(f"Sweeping to site [{site + 1}/{self.n_sites}], E0 = {1 / energy + self._offset}")
            self._env.update_mps(site, psi)
            self.perturb_wave_function(site)
            self._env.split_tensor(site, direction=direction)
            self._env.update(site, direction=direction)
            self._env2.update(site, direction=direction)
        return energy

    def run(self, tol: float = 1e-7, max_sweep: int = 100, metric: Metric = Metric.ENERGY, **kwargs) -> list[float]:
        """:386-395: sweeps on lambda, then 1/lambda + offset and the restored state."""
        lam = super().run(tol, max_sweep, metric, **kwargs)
        self._restore_mps()
        return (np.reciprocal(np.asarray(lam, dtype=float)) + self._offset).tolist()

    update = run

    @property
    def measurements(self) -> MatrixProductStateMeasurements:
        if len(self._energies) == 1:
            raise RuntimeError("FiniteDMRG is probably not executed yet.")
        return MatrixProductStateMeasurements(self.restored_mps)

    def variance(self) -> float:
        """<psi_r|(H - eps)^2|psi_r> - lambda^2 - offset^2 on the restored (unnormalised) state, as
        the reference computes it (:403-407)."""
        from .matrix_product_state import expectation_value

        return expectation_value(self.restored_mps, self._env.mpo.square()) - self._energies[-1] ** 2 - \
            self._offset ** 2


class BatchedFiniteDMRG:
    """Many independent chains of one shape (disorder realisations, parameter scans) swept in
    lockstep, every kernel spanning all chains: FiniteDMRG.run (finite_dmrg.py:214-257) per chain,
    computed as one stacked problem.

    Chain c starts from MatrixProductState.random(n, bond_dim, d, seed=seeds[c]) (default
    seeds: ``seed + c``) exactly as ``FiniteDMRG(mpos[c], bond_dim, seed=seeds[c])`` does, and
    each site update applies the reference's steps to every chain at once: the lowest eigenpair
    (dense Jacobi below ``exact_solver_dim`` elements, else the batched Davidson with a per-chain
    convergence mask; in batches of 64 chains or more, the last <= 1/64 of the chains stop after
    twice the expansions the rest needed and keep their best Ritz vector, counted in
    ``stats['unconverged']``), the 1e-5 perturbation, the QR gauge move and the environment update. A
    chain stops recording energies once its |dE| < tol (its ``energies`` end there, as in
    FiniteDMRG.run); the batch sweeps until every chain has converged or max_sweep.

    ``precision``: 'fp64' native FP64 GEMMs; 'mixed' (or 'df64') double-FP32 GEMMs on the FP32
    pipe (FP64-class products, ~2^-48 per product) for the matvecs, environment updates and
    gauge moves; the Rayleigh-Ritz, Gram-Schmidt and residuals stay FP64."""

    def __init__(self, mpos, bond_dim: int | None = None, *, chi: int | None = None, seed: int = 100,
                 seeds=None, precision: str = "fp64", exact_solver_dim: int = 200, max_iter: int = 400,
                 max_basis: int = 24, device=None):
        mpos = list(mpos)
        if not mpos:
            raise ValueError("BatchedFiniteDMRG needs at least one MPO")
        bond_dim = bond_dim if bond_dim is not None else chi
        if bond_dim is None:
            raise TypeError("BatchedFiniteDMRG needs bond_dim (or chi)")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        n, d = mpos[0].n_sites, mpos[0].phys_dim
        ws = [m.device_tensors(self.device) for m in mpos]
        for m, w in zip(mpos, ws):
            if m.n_sites != n or m.phys_dim != d or any(a.shape != b.shape for a, b in zip(w, ws[0])):
                raise ValueError("BatchedFiniteDMRG stacks chains of one shape (n, d, MPO bonds); use "
                                 "StreamedFiniteDMRG for mixed shapes")
        self.n_chains, self._n, self._d = len(mpos), n, d
        self._bond_dim = int(bond_dim)
        self.precision = precision
        K.precision_code(precision)
        self._exact_solver_dim = exact_solver_dim
        self.max_iter, self.max_basis = max_iter, max_basis
        seeds = list(seeds) if seeds is not None else [seed + c for c in range(self.n_chains)]
        if len(seeds) != self.n_chains:
            raise ValueError("one seed per chain")
        self.seeds = seeds
        # per site: stacked [B, ...] tensors
        self._w = [torch.stack([w[s] for w in ws]).contiguous() for s in range(n)]
        states = [MatrixProductState.random(n, self._bond_dim, d, seed=sd, device=self.device) for sd in seeds]
        self._t = [torch.stack([m.tensors[s] for m in states]).contiguous() for s in range(n)]
        del states
        B = self.n_chains
        one = torch.ones((B, 1, 1, 1), dtype=torch.float64, device=self.device)
        self._left = {0: one}
        self._right = {n - 1: one.clone()}
        for s in range(1, n):
            self._left[s] = K.batched_env_update(1, self._left[s - 1], self._t[s - 1], self._w[s - 1],
                                                 precision=self.precision)
        for s in range(n - 2, -1, -1):
            self._right[s] = K.batched_env_update(-1, self._right[s + 1], self._t[s + 1], self._w[s + 1],
                                                  precision=self.precision)
        self._energies: list[list[float]] = [[] for _ in range(B)]
        self.converged = [False] * B
        self.sweeps = [0] * B
        self.sweep_seconds: list[float] = []
        self.stats = {"dense_solves": 0, "iterative_solves": 0, "expansions": 0, "unconverged": 0}

    @property
    def n_sites(self) -> int:
        return self._n

    @property
    def bond_dim(self) -> int:
        return self._bond_dim

    @property
    def energies(self) -> list[list[float]]:
        return [list(e) for e in self._energies]

    def mps(self, chain: int) -> MatrixProductState:
        """Chain ``chain``'s MPS (copies of its site tensors)."""
        return MatrixProductState([t[chain].clone() for t in self._t], device=self.device)

    def _solve(self, site: int, tol: float) -> torch.Tensor:
        x = self._t[site]
        L, W, R = self._left[site], self._w[site], self._right[site]
        B = self.n_chains
        if x[0].numel() < self._exact_solver_dim:
            self.stats["dense_solves"] += 1
            H = K.batched_full_matrix1(L, W, R)
            evals, evecs = K.eigh_batched(list(H), keep=1)
            self._t[site] = evecs[:, : x[0].numel(), 0].reshape(x.shape).contiguous()
            return evals[:, 0]
        self.stats["iterative_solves"] += 1
        X = x.clone()
        evals, resid, its, active = K.batched_davidson1(L, W, R, X, tol=tol, max_iter=self.max_iter,
                                                        max_basis=self.max_basis, precision=self.precision)
        self.stats["expansions"] += its
        n_bad = int(active.sum().item())
        if n_bad:
            self.stats["unconverged"] += n_bad
            logger.warning(f"site {site}: {n_bad} of {B} chains' Davidson did not converge after {its} expansions")
        self._t[site] = X
        return evals

    def sweep(self, direction: Direction = Direction.RIGHTWARD, tol: float = 1e-8) -> torch.Tensor:
        """One sweep of every chain (finite_dmrg.py:143-171); returns each chain's last local
        energy (device tensor [B])."""
        n = self._n
        sites = range(n - 1) if direction == Direction.RIGHTWARD else range(n - 1, 0, -1)
        e = None
        for site in sites:
            e = self._solve(site, tol)
            psi = self._t[site]
            hpsi = K.batched_matvec1(self._left[site], self._w[site], self._right[site], psi,
                                     precision=self.precision)
            psi.add_(hpsi, alpha=1e-5)
            if direction == Direction.RIGHTWARD:
                K.batched_gauge_move(1, self._t[site], self._t[site + 1], precision=self.precision)
                self._left[site + 1] = K.batched_env_update(1, self._left[site], self._t[site], self._w[site],
                                                            precision=self.precision)
            else:
                K.batched_gauge_move(-1, self._t[site], self._t[site - 1], precision=self.precision)
                self._right[site - 1] = K.batched_env_update(-1, self._right[site], self._t[site], self._w[site],
                                                             precision=self.precision)
        return e

    def run(self, tol: float = 1e-8, max_sweep: int = 100, metric: Metric = Metric.ENERGY) -> list[list[float]]:
        """Sweep all chains until each has |dE| < tol (per chain) or ``max_sweep`` sweeps;
        returns every chain's per-sweep energies up to its convergence."""
        if metric != Metric.ENERGY:
            raise NotImplementedError("batched chains converge on the energy metric")
        for n_sweep, direction in zip(range(1, max_sweep + 1), cycle([Direction.RIGHTWARD, Direction.LEFTWARD])):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e = self.sweep(direction, tol=tol).cpu().numpy()
            self.sweep_seconds.append(time.perf_counter() - t0)
            for c in range(self.n_chains):
                if self.converged[c]:
                    continue
                self._energies[c].append(float(e[c]))
                self.sweeps[c] = n_sweep
                if len(self._energies[c]) >= 2 and abs(self._energies[c][-1] - self._energies[c][-2]) < tol:
                    self.converged[c] = True
            if all(self.converged):
                break
        return self.energies


class StreamedFiniteDMRG:
    """Many independent chains of any shapes swept concurrently on CUDA streams (for chains that
    BatchedFiniteDMRG cannot stack because their sizes differ).

    Each chain is a ``FiniteDMRG`` built and swept on its own CUDA stream by one of ``workers``
    host threads (chain c on worker c mod workers). Every library call releases the GIL and a
    Davidson solve blocks only the thread that issued it, so the small kernels of different
    chains overlap on the GPU instead of leaving it idle between launches. Each chain's
    arithmetic does not depend on the stream it runs on: ``energies[c]`` equals
    ``FiniteDMRG(mpos[c], bond_dim, **kwargs).run(tol, max_sweep)`` for the same arguments.
    """

    def __init__(self, mpos, bond_dim: int | None = None, *, chi: int | None = None, workers: int = 8,
                 device=None, **kwargs):
        self._mpos = list(mpos)
        if not self._mpos:
            raise ValueError("StreamedFiniteDMRG needs at least one MPO")
        self._bond_dim = bond_dim if bond_dim is not None else chi
        if self._bond_dim is None:
            raise TypeError("StreamedFiniteDMRG needs bond_dim (or chi)")
        self._kwargs = kwargs
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.workers = max(1, min(int(workers), len(self._mpos)))
        self._streams = [torch.cuda.Stream(self.device) for _ in range(self.workers)]
        self.chains: list[FiniteDMRG | None] = [None] * len(self._mpos)
        self.sweeps: list[int] = [0] * len(self._mpos)
        self._map(self._build)

    def _map(self, fn):
        def work(w: int):
            torch.cuda.set_device(self.device)
            with torch.cuda.stream(self._streams[w]):
                for c in range(w, len(self._mpos), self.workers):
                    fn(c)
            self._streams[w].synchronize()

        with ThreadPoolExecutor(max_workers=self.workers) as ex:
            for fut in [ex.submit(work, w) for w in range(self.workers)]:
                fut.result()  # re-raises a chain's exception in the caller

    def _build(self, c: int):
        self.chains[c] = FiniteDMRG(self._mpos[c], self._bond_dim, device=self.device, **self._kwargs)

    def run(self, tol: float = 1e-8, max_sweep: int = 100, metric: Metric = Metric.ENERGY) -> list[list[float]]:
        """Sweep every chain until its own |dE| < tol or ``max_sweep`` (FiniteDMRG.run per chain,
        variance not computed). Returns the per-sweep energies of every chain."""

        def one(c: int):
            f = self.chains[c]
            for n_sweep, direction in zip(range(1, max_sweep + 1), cycle([Direction.RIGHTWARD, Direction.LEFTWARD])):
                f._energies.append(f.sweep(direction, tol=tol))
                f._variances.append(np.nan)
                self.sweeps[c] = n_sweep
                if f._converged(n_sweep, tol, max_sweep, metric):
                    break

        self._map(one)
        return self.energies

    def sweep(self, direction: Direction = Direction.RIGHTWARD, tol: float = 1e-8) -> list[float]:
        """One sweep of every chain in ``direction``; returns each chain's last local energy."""
        out = [0.0] * len(self._mpos)

        def one(c: int):
            out[c] = self.chains[c].sweep(direction, tol=tol)

        self._map(one)
        return out

    @property
    def energies(self) -> list[list[float]]:
        return [f.energies for f in self.chains]
