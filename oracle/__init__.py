"""CPU FP64 restatement of tnpy's DMRG / tSDRG path -- TEST INFRASTRUCTURE ONLY.

This package is the oracle that the CUDA path is checked against. It is a
plain numpy/scipy restatement of the reference algorithms (tanlin2013/tnpy),
written from their behaviour; every function cites the reference file:line it
follows. The reference itself cannot be imported here (quimb 1.4.0, primme
3.2.1 and tensornetwork 0.4.6 are absent), so:

* quimb tensor contractions are restated as explicit ``np.tensordot`` chains
  with quimb's index-order semantics (open indices in order of appearance;
  ``fuse`` moves fused groups to the front, row-major);
* ``primme.eigsh(which='SA')`` is restated with ``scipy.sparse.linalg.eigsh``
  (ARPACK) run at a tight tolerance;
* the unseeded ``quimb.MPS_rand_state`` is replaced with a seeded N(0, 1) MPS,
  right-canonicalised so that the first (rightward) sweep starts at an
  orthogonality centre on site 0.

Parity is pinned by the reference's own known-answer tests (exact
Hamiltonians, ED spectra, tSDRG block Hamiltonian and projector, the notebook
ED spectrum) through ``tests/golden/golden.json``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this package, and only as
the checker or as the timed CPU baseline -- never as part of the product path.
"""

from . import models, operators, mps, dmrg, tsdrg, ed  # noqa: F401
