"""FiniteDMRG's host-side sweep loop and convergence rule without a GPU
(finite_dmrg.py:173-257): directions alternate from a rightward first sweep, the run stops
once |dE| < tol or after max_sweep sweeps, the energies of every sweep are returned, and the
reference's warnings are logged. Sweeps are scripted; nothing touches the device."""
import logging

import numpy as np
import pytest
import torch

from tnpy_gb300.finite_dmrg import Direction, FiniteDMRG, Metric


def _scripted(energies, monkeypatch):
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    f = FiniteDMRG.__new__(FiniteDMRG)  # no environments: the loop logic only
    f._energies, f._variances, f.sweep_seconds = [np.nan], [np.nan], []
    f.compute_variance = False
    f.directions = []
    it = iter(energies)

    def sweep(direction, tol=1e-8, **kwargs):
        f.directions.append(direction)
        return next(it)

    f.sweep = sweep
    return f


def test_run_stops_at_tolerance(monkeypatch):
    f = _scripted([-1.0, -1.5, -1.5 - 1e-12, -9.0], monkeypatch)
    assert f.run(tol=1e-8, max_sweep=10) == [-1.0, -1.5, -1.5 - 1e-12]
    assert f.directions == [Direction.RIGHTWARD, Direction.LEFTWARD, Direction.RIGHTWARD]
    assert len(f.sweep_seconds) == 3


def test_update_is_run(monkeypatch):
    f = _scripted([-1.0, -1.0], monkeypatch)
    assert f.update(tol=1e-8, max_sweep=5) == [-1.0, -1.0]


def test_run_stops_at_max_sweep_with_warning(monkeypatch, caplog):
    f = _scripted([-1.0, -2.0, -3.0, -4.0], monkeypatch)
    with caplog.at_level(logging.WARNING, logger="tnpy"):
        assert f.run(tol=1e-8, max_sweep=3) == [-1.0, -2.0, -3.0]
    assert any("Maximum number of sweeps 3 is reached" in r.getMessage() for r in caplog.records)


def test_large_decrease_logs_the_local_minimum_warning(monkeypatch, caplog):
    f = _scripted([-1.0, -2.0, -2.0], monkeypatch)
    with caplog.at_level(logging.WARNING, logger="tnpy"):
        f.run(tol=1e-8, max_sweep=5)
    assert any("Might be trapped in local minimum" in r.getMessage() for r in caplog.records)


def test_converged_rule_matches_reference_cases():
    f = FiniteDMRG.__new__(FiniteDMRG)
    f._energies = [np.nan, -1.0]
    assert not f._converged(1, 1e-8, 10, Metric.ENERGY)  # first sweep: gradient is NaN
    f._energies = [np.nan, -1.0, -1.0 + 5e-9]
    assert f._converged(2, 1e-8, 10, Metric.ENERGY)
    f._energies = [np.nan, -1.0, -1.0 + 5e-6]  # energy went up by more than tol: keep sweeping
    assert not f._converged(2, 1e-8, 10, Metric.ENERGY)
    f._variances = [np.nan, 1e-3, 1e-3 - 1e-12]
    assert f._converged(2, 1e-8, 10, Metric.VARIANCE)


def test_measurements_need_a_run():
    f = FiniteDMRG.__new__(FiniteDMRG)
    f._energies = [np.nan]
    with pytest.raises(RuntimeError):
        _ = f.measurements


class _FakeSolverSite:
    """Stands in for the device pieces of one_site_solver: a site tensor, an environment whose
    site_operator returns placeholders, and a scripted davidson1."""

    def __init__(self, results, monkeypatch, stats=None):
        import tnpy_gb300.kernels as K

        self.calls = []
        self.anchored = []
        it = iter(results)
        st = iter(stats or [])

        def davidson1(L, W, R, x, tol=1e-8, max_iter=200, max_basis=24, precision="fp64", raise_on_fail=False,
                      start_anchored=False):
            self.calls.append(precision)
            self.anchored.append(start_anchored)
            return next(it)

        monkeypatch.setattr(K, "davidson1", davidson1)
        monkeypatch.setattr(K, "davidson1_stats",
                            lambda: next(st, {"phase1": 3, "anchored": 2, "anchors": 1, "restarts": 0}))
        f = FiniteDMRG.__new__(FiniteDMRG)
        f._settled = {}
        f._exact_solver_dim = 200
        f.max_iter, f.max_basis = 400, 24
        f.stats = {"matvecs": 0, "dense_solves": 0, "iterative_solves": 0, "unconverged": 0, "df64_retries": 0}

        class _Env:
            mps = type("M", (), {"tensors": [torch.zeros((16, 2, 16), dtype=torch.float64)]})()

            def site_operator(self, site):
                return None, None, None

        f._env = _Env()
        self.f = f


def test_unconverged_mixed_solve_is_continued_in_fp64_class(monkeypatch, caplog):
    s = _FakeSolverSite([(-1.0, 0.5, 16, False), (-1.2, 1e-9, 30, True)], monkeypatch)
    s.f.precision = "mixed"
    with caplog.at_level(logging.INFO, logger="tnpy"):
        e, _ = s.f.one_site_solver(0, 1e-8)
    assert e == -1.2 and s.calls == ["mixed", "df64"]
    assert s.f.stats["df64_retries"] == 1 and s.f.stats["unconverged"] == 0 and s.f.stats["matvecs"] == 46
    assert not any(r.levelno >= logging.WARNING for r in caplog.records)


def test_unconverged_solve_warns_every_time(monkeypatch, caplog):
    s = _FakeSolverSite([(-1.0, 0.5, 400, False)] * 2, monkeypatch)
    s.f.precision = "fp64"
    with caplog.at_level(logging.WARNING, logger="tnpy"):
        s.f.one_site_solver(0, 1e-8)
        s.f.one_site_solver(0, 1e-8)
    warned = [r for r in caplog.records if "did not converge" in r.getMessage()]
    assert len(warned) == 2 and s.f.stats["unconverged"] == 2


def test_unconverged_solve_can_raise(monkeypatch):
    s = _FakeSolverSite([(-1.0, 0.5, 400, False)], monkeypatch)
    s.f.precision = "fp64"
    with pytest.raises(RuntimeError):
        s.f.one_site_solver(0, 1e-8, raise_on_fail=True)


def test_settled_site_starts_at_the_anchor(monkeypatch):
    """A mixed solve that converged at its first anchor with no split-BF16 expansion marks its
    site settled; the next solve there starts with the anchor (start_anchored), and a solve that
    needed more clears the mark."""
    settled = {"phase1": 1, "anchored": 0, "anchors": 1, "restarts": 0}
    busy = {"phase1": 6, "anchored": 3, "anchors": 2, "restarts": 0}
    s = _FakeSolverSite([(-1.0, 1e-9, 1, True), (-1.0, 1e-9, 0, True), (-1.0, 1e-9, 9, True),
                         (-1.0, 1e-9, 9, True)], monkeypatch,
                        stats=[settled, dict(settled, phase1=0), busy, busy])
    s.f.precision = "mixed"
    for _ in range(4):
        s.f.one_site_solver(0, 1e-8)
    assert s.anchored == [False, True, True, False]
    assert s.f.stats["anchored_starts"] == 2
