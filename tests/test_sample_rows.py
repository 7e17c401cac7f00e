"""The rows the bench's accuracy check compares (CPU).

`bench.py` checks the device plan of a full workload against the FP64 oracle on the CPU
sample that `oracle/cpu_baseline.py` times: the first wave, a subset ``f_idx`` of the
frequencies and the first ``n_mix`` receive mixes.  Observation rows are ordered
measurement -> mix -> frequency, so the sample's row (m, j) is the full operator's row
m * F + f_idx[j] of wave 0.  This pins that mapping on small oracle configurations: the
sample operator's forward rows equal those rows of the full operator, and the adjoint of
the full operator fed only those rows equals the sample operator's adjoint.
"""

import dataclasses

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, configs, forward_quick_cpu


@pytest.mark.parametrize("name,n_freq,n_mix", [("c1", 3, 5), ("c2", 2, 3)])
def test_sample_rows_are_rows_of_the_full_operator(name, n_freq, n_mix):
    cfg = configs.small_config(name)
    full = configs.build(cfg)
    F = len(cfg.f)
    f_idx = np.linspace(0, F - 1, n_freq).round().astype(int)
    scfg = dataclasses.replace(cfg, f=cfg.f[f_idx], waves=cfg.waves[:1])
    samp = configs.build(scfg)
    meas = [dataclasses.replace(m, mixes=m.mixes[:n_mix]) for m in samp.op.measurements]
    sop = dataclasses.replace(samp.op, measurements=meas)
    rng = np.random.default_rng(3)
    gamma = rng.standard_normal((cfg.setup.n_points, 2))
    u_s = forward_quick_cpu(sop, gamma)
    rows = np.array([m * F + fi for m in range(n_mix) for fi in f_idx])
    u_f = forward_quick_cpu(full.op, gamma)
    assert u_s.shape == (len(rows), 2)
    assert np.max(np.abs(u_f[rows] - u_s)) <= 1e-12 * np.max(np.abs(u_s))
    u_in = np.zeros((full.op.n_observations, 2), dtype=complex)
    u_in[rows] = u_s
    g_f = adjoint_quick_cpu(full.op, u_in)
    g_s = adjoint_quick_cpu(sop, u_s)
    assert np.max(np.abs(g_f - g_s)) <= 1e-12 * np.max(np.abs(g_s))
