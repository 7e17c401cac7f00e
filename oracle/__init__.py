"""FP64 CPU oracle for the Born scattering operator.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
C-ABI or the Python host mirror) imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` use it, and only as the checker or the timed CPU
baseline.

The package restates, in numpy/scipy FP64, the reference toolbox's
(mschiffn/comp_ui_toolbox) CPU Born operator and the table builders that
feed it.  Every function cites the reference file:line it follows.

Parity status: the reference is MATLAB-only and none of its scripts pin
numbers on this path (no golden vectors, no fixtures, no asserts), so the
restatement is checked against mathematics (mpmath Hankel functions at 30
digits, the dot-product adjointness test, the reference's own symmetric-grid
index map against direct per-element evaluation) rather than against outputs
of the reference itself: parity unpinned.
"""

from .born_oracle import *  # noqa: F401,F403
