"""ORACLE — test infrastructure, not product code.

A CPU restatement of the reference ionization library's mesh time-evolution
path (JoshKarpel/ionization v0.2.0), used for three things only:

  * the parity checker in ``tests/`` and ``__graft_entry__.smoke()``;
  * the timed CPU baseline (``bench.py`` ``cpu_baseline`` leg and the
    ``--impl reference`` arm);
  * nothing else.  The product package ``ionization_gb300`` never imports,
    links or executes anything here; its compute path is CUDA only.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against fixtures produced by running the reference itself
(``tests/golden/make_golden.py``).

Contents
  tdma.c        Thomas solver, restating ionization/cy.pyx:9-50
  _lib.py       gcc build + ctypes binding of tdma.c
  physics.py    pulses, potentials, masks, states (host FP64 formulas)
  mesh.py       grids, operator diagonals, evolution sequences, run loop
"""

from . import physics, mesh  # noqa: F401
from ._lib import tdma, tdma_batched, tdma_from_dia, build  # noqa: F401
