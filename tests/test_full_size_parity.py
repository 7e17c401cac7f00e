"""Full-size parity against the FP64 oracle on stratified samples of every workload (GPU).

The device plan is the full benchmark plan (2d-plain 256^2 x 64 f; 2d-gradient 512^2 x 192 f x
11 waves, absorbing; 2d-batched 512^2 x 128 f x 16 waves -> 32 mixes; 3d 128^3 x 64 f x 1024
elements with the stored, streamed and generated table; the first problem of the uneven LASSO
batch).  The oracle (``forward_quick_cpu`` / ``adjoint_quick_cpu``, ``operator_born.m:332-596``)
evaluates a stratified sample (``tests/full_size_oracle.py``): the first, middle and last wave,
four frequencies including the top of the band (largest k r), four receive mixes, every element,
the full grid (3d: its first four axial planes).  Checks, per column of 4 seeded objects:

* forward: the sample's rows of the device output for the workload's seeded sparse gamma
  (supported on the sample's grid planes);
* adjoint: the device adjoint of an observation vector that is nonzero on exactly the sample's
  rows, against the oracle adjoint of those rows, on every point of the sample's grid.

Bound: relative L2 <= 1e-5 for every output and path (FP32 CUDA cores; split-BF16 tcgen05 over
slots and elements; split-BF16 GEMMs against the folded operator).  With CUI_PARITY_REPORT set to a
file name the measured errors are appended there as JSON lines.
"""

from __future__ import annotations

import json
import os

import numpy as np
import pytest

from tests.full_size_oracle import adjoint_parallel, full_rows, sample_operator
from tests.helpers import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5
B = 4
_REF = {}


def oracle_config(name):
    from comp_ui_toolbox_gb300.workloads import lasso_problem, workload
    from oracle import configs
    if name == "2d-lasso[0]":
        w = lasso_problem(0)
        s = configs._setup_2d(w.n_points_axis[0], w.n_points_axis[1], w.n_elements, configs.LOSSLESS)
        return configs.BornConfig(w.name, s, np.asarray(w.f), [configs.Wave("qpw", a) for _, a in w.waves],
                                  density=w.density, seed=w.seed), w
    return configs.config({"2d-plain": "c0", "2d-gradient": "c1", "2d-batched": "c2", "3d": "c3"}[name]), workload(name)


def reference(name):
    """Sample rows, gamma and the oracle's forward and adjoint (cached per workload)."""
    if name in _REF:
        return _REF[name]
    from oracle import adjoint_quick_cpu, forward_quick_cpu
    cfg, w = oracle_config(name)
    n_planes = 4 if name == "3d" else None
    op, w_idx, f_idx, m_idx, M = sample_operator(cfg, n_planes)
    rows = full_rows(w_idx, m_idx, f_idx, M, len(w.f))
    Ps = op.setup.n_points
    gamma = np.zeros((w.n_points, B))
    gamma[:Ps] = w.gamma(seed=w.seed + 7, n_objects=B)[:Ps].real
    u_ref = forward_quick_cpu(op, gamma[:Ps])
    rng = np.random.default_rng(11)
    y = rng.standard_normal((len(rows), B)) + 1j * rng.standard_normal((len(rows), B))
    if name == "2d-batched":  # 12 (wave, mix) blocks x 128 elements over the full grid: a spawn pool
        g_ref = adjoint_parallel(cfg, n_planes, op, y)
    else:
        g_ref = adjoint_quick_cpu(op, y)
    _REF[name] = dict(w=w, rows=rows, Ps=Ps, gamma=gamma, u_ref=u_ref, y=y, g_ref=g_ref)
    return _REF[name]


CASES = [("2d-plain", "fp32", "auto"), ("2d-plain", "bf16x3", "auto"),
         ("2d-gradient", "fp32", "auto"), ("2d-gradient", "bf16x3", "auto"),
         ("2d-batched", "fp32", "auto"), ("2d-batched", "bf16x3", "auto"), ("2d-batched", "bf16x3-folded", "auto"),
         ("3d", "fp32", "stored"), ("3d", "fp32", "streamed"), ("3d", "fp32", "generated"),
         ("2d-lasso[0]", "fp32", "auto"), ("2d-lasso[0]", "bf16x3", "auto")]


@pytest.mark.parametrize("name,precision,storage", CASES)
def test_full_size_matches_oracle_sample(name, precision, storage):
    from comp_ui_toolbox_gb300 import OperatorBorn
    r = reference(name)
    w = r["w"]
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=B, table_storage=storage)
    op.set_precision(precision)
    u = op.forward(torch.from_numpy(r["gamma"].astype(np.complex64)).cuda()).cpu().numpy()[r["rows"]]
    u_in = np.zeros((op.n_observations, B), dtype=np.complex64)
    u_in[r["rows"]] = r["y"]
    g = op.adjoint(torch.from_numpy(u_in).cuda()).cpu().numpy()[: r["Ps"]]
    assert op.device_status() == 0
    op.close()
    errs = {"forward": [rel_l2(u[:, k], r["u_ref"][:, k]) for k in range(B)],
            "adjoint": [rel_l2(g[:, k], r["g_ref"][:, k]) for k in range(B)]}
    if os.environ.get("CUI_PARITY_REPORT"):
        with open(os.environ["CUI_PARITY_REPORT"], "a") as fh:
            fh.write(json.dumps({"workload": name, "precision": precision, "table_storage": storage,
                                 "rows": int(len(r["rows"])), "points": int(r["Ps"]), "columns": B,
                                 "rel_l2_forward_max": max(errs["forward"]),
                                 "rel_l2_adjoint_max": max(errs["adjoint"])}) + "\n")
    assert max(errs["forward"]) <= TOL, errs
    assert max(errs["adjoint"]) <= TOL, errs
