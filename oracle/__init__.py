"""FP64 CPU oracle for the Born scattering operator.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library, its
C-ABI or the Python host mirror) imports this package.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` use it, and only to check the library's results or as
the timed CPU baseline.

The package restates, in numpy/scipy FP64, the reference toolbox's
(mschiffn/comp_ui_toolbox) CPU Born operator and the table builders that
feed it.  Every function cites the reference file:line it follows.

Parity status: pinned against the reference itself.  The reference's MEX
gateway ``+scattering/combined_quick_gpu.cu`` compiles unchanged on the host
against the stub MEX and CUDA runtimes of ``oracle/ref_mex`` (its device kernel
``compute_matrix_kernel``, ``:1099-1124``, runs as a host restatement, and
``cublasCgemm`` as a host FP32 complex GEMM).  Its outputs on the small
configurations are frozen in ``tests/golden/reference_gateway.npz``
(``tests/golden/make_reference_golden.py``), and the oracle agrees with them to
FP32 rounding (relative L2 <= 1e-6; ``tests/test_reference_pinning.py``).  The
restatement is also checked against mathematics: mpmath Hankel functions at 30
digits, the dot-product adjointness test, and the reference's symmetric-grid
index map against direct per-element evaluation.
"""

from .born_oracle import *  # noqa: F401,F403
