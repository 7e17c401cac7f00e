"""Generate the small golden fixtures of the Born operator from the FP64 oracle.

The reference (MATLAB) cannot run without MATLAB and its scripts pin
no numbers on this path, so these fixtures are oracle outputs: they freeze
the restatement (tables, incident fields, forward and adjoint) so that any
drift of the oracle is caught, and they give the CPU suite known answers.

Run from the repository root:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import Absorption, Setup, adjoint_quick_cpu, forward_quick_cpu  # noqa: E402
from oracle import configs  # noqa: E402

OUT = Path(__file__).resolve().parent / "born_tiny.npz"


def tiny_config() -> configs.BornConfig:
    s = Setup(n_points_axis=(20, 6), delta_axis=(1e-4, 1e-4), z_start=2e-3, n_elements_axis=(4,),
              pitch_axis=(2e-4,), width_axis=(1.8e-4,), n_face_axis=(2,),
              absorption=Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True))
    return configs.BornConfig("tiny", s, np.linspace(3e6, 5e6, 3),
                              [configs.Wave("qpw", (-5.0,)), configs.Wave("rad", seed=3)],
                              mixing="pm1", n_mixes=3, mix_seed=4, n_objects=2, density=0.2, seed=5)


def generate():
    cfg = tiny_config()
    b = configs.build(cfg, direct_elements=True)
    gamma = configs.make_gamma(cfg, complex_values=True)
    u = forward_quick_cpu(b.op, gamma)
    rng = np.random.default_rng(6)
    y = rng.standard_normal(u.shape) + 1j * rng.standard_normal(u.shape)
    g = adjoint_quick_cpu(b.op, y)
    return dict(table_rx=b.table_rx, p_in_0=b.op.measurements[0].p_incident,
                p_in_1=b.op.measurements[1].p_incident, h_ref=b.op.h_ref, shift=b.op.shift,
                gamma=gamma, u=u, y=y, gamma_hat=g)


if __name__ == "__main__":
    np.savez_compressed(OUT, **generate())
    print(OUT, OUT.stat().st_size, "bytes")
