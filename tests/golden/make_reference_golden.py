"""Golden vectors produced by the reference's own code: the MEX gateway
``+scattering/combined_quick_gpu.cu`` (``mexFunction``, modes 1 = forward and 2 = adjoint),
compiled unchanged and run on the host by ``oracle/ref_mex`` (host stand-ins of the MEX
runtime, the CUDA runtime and cuBLAS; the one device kernel, ``compute_matrix_kernel``, as a
host restatement of its formula in FP32).

For each small configuration whose field of view is at least as wide as the array (where the
reference's ``indices_grid_FOV_shift`` is valid) the fixture holds the operator inputs'
checksums, seeded complex and real gamma columns with the gateway's forward outputs, and seeded
observation columns with the gateway's adjoint outputs.  The gateway computes in FP32, so its
outputs are stored as complex64 without loss.

Needs the reference checkout (this machine); the fixture it writes is what the tests read:

    python tests/golden/make_reference_golden.py
"""

from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import configs  # noqa: E402
from oracle.ref_mex import build as ref_build  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_gateway.npz"
CONFIGS = ("c1", "c2", "ragged", "c3")


def table_checksums(b: configs.BuiltOperator) -> np.ndarray:
    """Sums that identify the operator the oracle builds for a configuration."""
    op = b.op
    return np.array([np.abs(op.h_ref).sum(), float(np.asarray(op.shift).sum()),
                     sum(np.abs(m.p_incident).sum() for m in op.measurements),
                     sum(np.abs(mx.pref).sum() for m in op.measurements for mx in m.mixes)])


def generate():
    lib = ref_build.build()
    if lib is None:
        raise SystemExit("the reference checkout is not available: nothing to generate")
    from oracle.ref_runner import ReferenceGateway
    gw = ReferenceGateway(lib)
    src = ref_build.reference_source()
    out = {"source_sha256": np.frombuffer(hashlib.sha256(src.read_bytes()).digest(), dtype=np.uint8),
           "configs": np.array(CONFIGS)}
    for name in CONFIGS:
        b = configs.build(configs.small_config(name))
        assert b.op.h_ref is not None, name
        B = max(2, b.cfg.n_objects)
        rng = np.random.default_rng(900 + CONFIGS.index(name))
        gamma = configs.make_gamma(b.cfg, n_objects=B, seed=500 + CONFIGS.index(name), complex_values=True)
        gamma_real = rng.standard_normal((b.op.setup.n_points, 1)) * (rng.random((b.op.setup.n_points, 1)) < 0.2)
        y = rng.standard_normal((b.op.n_observations, B)) + 1j * rng.standard_normal((b.op.n_observations, B))
        node = gw.operator(b.op)
        out[f"{name}/checksums"] = table_checksums(b)
        out[f"{name}/gamma"] = gamma
        out[f"{name}/u"] = gw.call(node, 1, gamma).astype(np.complex64)
        out[f"{name}/gamma_real"] = gamma_real
        out[f"{name}/u_real"] = gw.call(node, 1, gamma_real).astype(np.complex64)
        out[f"{name}/y"] = y
        out[f"{name}/gamma_hat"] = gw.call(node, 2, y).astype(np.complex64)
        gw.reset()
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **generate())
    print(OUT, OUT.stat().st_size, "bytes")
