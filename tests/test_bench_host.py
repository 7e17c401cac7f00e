"""Host-side logic of ``bench.py`` (CPU, no device call): the roofline block for every
workload, contraction path and table storage the bench can report, and the size of a
stored table."""

import argparse
import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import bench
    return bench


def test_full_table_bytes():
    bench = _bench()
    from comp_ui_toolbox_gb300.workloads import workload
    assert bench.full_table_bytes(workload("3d")) == 64 * 128 * 221 * 221 * 8
    assert bench.full_table_bytes(workload("2d-batched")) == 128 * 512 * (512 + 127 * 4) * 8


@pytest.mark.parametrize("name,precision,storage", [
    ("2d-batched", "bf16x3-folded", "stored"),
    ("2d-batched", "bf16x3", "stored"),
    ("2d-batched", "fp32", "stored"),
    ("2d-gradient", "bf16x3", "stored"),
    ("2d-plain", "fp32", "stored"),
    ("3d", "fp32", "stored"),
    ("3d", "fp32", "streamed"),
    ("3d", "fp32", "generated"),
])
def test_roofline_block(name, precision, storage):
    bench = _bench()
    from comp_ui_toolbox_gb300.workloads import workload
    w = workload(name)
    n_dims = len(w.n_points_axis)
    full = bench.full_table_bytes(w)
    args = argparse.Namespace(workload=name, precision=precision, n_freq_used=len(w.f), table_used=storage,
                              n_dims=n_dims, full_table_bytes=full)
    table_bytes = {"stored": full, "streamed": full // 6, "generated": 0}[storage]
    info = {"contraction_macs": 6.87e10, "channel_macs": 1.72e10, "n_points": w.n_points, "n_observations": 65536,
            "table_bytes": table_bytes, "incident_bytes": 4 * 10**9, "folded_bytes": 65536 * w.n_points * 8}
    kt = {"ms_forward": 70.0, "n_forward": 1, "ms_adjoint": 60.0, "n_adjoint": 1}
    B = 64 if name == "2d-batched" else 1
    r = bench.roofline_of(args, info, kt, B, {"sm_mhz": 2070.0}, p_used=0.857)
    json.dumps(r)  # the block goes into the JSON line as is
    assert r["bound"] == {"bf16x3": "tensor", "bf16x3-folded": "hbm"}.get(precision, "fp32")
    assert r["frac"] > 0 and r["achieved"] > 0 and r["peak"] > 0
    # algorithmic work: the channel-contraction entries, over the forward's occupied points
    assert r["work"]["algorithmic_complex_macs_per_launch"] == pytest.approx(1.72e10 * B * 0.857)
    if precision == "bf16x3-folded":
        assert r["kernel"] == "phi_gemm_kernel<false>"
        assert r["hbm"]["compulsory_bytes"] >= info["folded_bytes"]
        assert r["tensor"]["frac"] == pytest.approx(24 * 1.72e10 * B * 0.857 / 0.070 / 1e12 / r["tensor"]["peak"])
        return
    assert r["hbm"]["compulsory_bytes"] >= info["incident_bytes"]
    expected = {("bf16x3", 2): "fwd_tc2_kernel", ("fp32", 2): "fwd_dense_kernel"}.get((precision, n_dims))
    if n_dims == 3:
        expected = "fwd_gen_kernel" if storage == "generated" else "fwd_dense3_kernel"
    assert r["kernel"] == expected  # the forward dominates (70 ms vs 60 ms)
    if storage == "streamed":  # the full table is written by the chunk generator and read back
        assert r["hbm"]["compulsory_bytes"] >= 2 * full
