"""bench.py's CPU legs without a GPU: the reference arm is a measurement of real site updates
of the CPU restatement (no modelled matvec counts), and its line keeps the bench contract."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_sweep_site_weight_counts_full_chi_equivalents():
    import bench

    # 80 of the 99 sites of XXZ(100) at chi=1024 have full bonds; the edges add ~1.1
    assert abs(bench.sweep_site_weight(100, 1024) - 81.142857) < 1e-5
    # chi above every bond: weights of the exact-size chain
    assert bench.sweep_site_weight(4, 64) == (1 * 2 * 2 + 2 * 4 * 4 + 4 * 2 * 4) / 64**3


def test_bulk_pair_site_updates_settle_variationally():
    """Bouncing between two bulk sites is a sweep restricted to them: the energies settle, and
    they stay above the lowest eigenvalue of the two-site effective Hamiltonian in the fixed
    environments (the one-site updates keep the bond between the two sites at its size)."""
    import argparse

    import bench

    a = argparse.Namespace(n=12, chi=8, delta=-0.5, seed=3, tol=1e-10)
    L, Wi, Wj, R, ai, aj = bench.cpu_pair_from_random_mps(a)
    pair = bench.CpuBulkPair(L, Wi, Wj, R, ai, aj, tol=1e-12)
    es = [pair.step()[0] for _ in range(16)]
    assert abs(es[-1] - es[-2]) < 1e-8 * abs(es[-1])
    h = np.einsum("awx,wvst,vuqr,cuy->asqcxtry", L, Wi, Wj, R)
    n = L.shape[0] * 2 * 2 * R.shape[0]
    e2 = np.linalg.eigvalsh(h.reshape(n, n))[0]
    assert es[-1] >= e2 - 1e-10 and es[-1] - e2 < 1e-2 * abs(e2), (es[-1], e2)


def test_reference_arm_line_is_a_measurement():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", "16", "--chi", "32",
                          "--steps", "3", "--warmup", "1"], capture_output=True, text=True, timeout=300,
                         cwd=str(ROOT))
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "sweeps/s" and line["steps"] == 3
    cb = line["cpu_baseline"]
    assert cb["site_updates_timed"] == 3 and cb["kind"] == "port"
    # value follows from the timed site updates and the sweep's site weight only
    assert abs(line["value"] - 1.0 / (cb["seconds_per_site_update"] * cb["sweep_site_weight"])) < 1e-9 * line["value"]
    assert abs(line["ms_per_step"] - 1e3 * cb["seconds_per_site_update"]) < 1e-6
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
