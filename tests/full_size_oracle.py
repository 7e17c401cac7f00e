"""FP64 oracle references for stratified samples of the full-size workloads (test helper).

A sample keeps the full grid (or, for the 3D workload, its first axial planes), every element,
and a stratified subset of the workload's incident waves (first, middle, last), frequencies
(lowest, two inner, the top of the band, where k r is largest) and receive mixes (first, two
inner, last).  Its operator is built by the oracle (``oracle.configs``) from the workload's
configuration with the excitation spectrum of the full band, so its rows are rows of the
full-size operator: row (w, m, f) of the full plan is ``(w * M + m) * F + f``.
"""

from __future__ import annotations

import dataclasses
import multiprocessing as mp
import os

import numpy as np

_STATE = {}


def pick(n: int, k: int) -> list:
    """k indices spread over range(n), first and last included."""
    return sorted(set(int(round(i * (n - 1) / max(1, k - 1))) for i in range(k)))


def sample_config(cfg, n_planes=None):
    W, F = len(cfg.waves), len(cfg.f)
    w_idx, f_idx = pick(W, 3), pick(F, 4)
    cfg = dataclasses.replace(cfg)
    cfg.band = (float(np.min(cfg.f)), float(np.max(cfg.f)))
    cfg.f = np.asarray(cfg.f)[f_idx]
    cfg.waves = [cfg.waves[i] for i in w_idx]
    if n_planes is not None:
        ax = tuple(cfg.setup.n_points_axis)
        cfg.setup = dataclasses.replace(cfg.setup, n_points_axis=ax[:-1] + (min(n_planes, ax[-1]),))
    return cfg, w_idx, f_idx


def sample_operator(cfg, n_planes=None):
    """(restricted OperatorTables, wave indices, frequency indices, mix indices, mixes per wave)."""
    from oracle import configs
    scfg, w_idx, f_idx = sample_config(cfg, n_planes)
    b = configs.build(scfg)
    M = len(b.op.measurements[0].mixes)
    m_idx = pick(M, 4)
    meas = [dataclasses.replace(m, mixes=[m.mixes[i] for i in m_idx]) for m in b.op.measurements]
    return dataclasses.replace(b.op, measurements=meas), w_idx, f_idx, m_idx, M


def full_rows(w_idx, m_idx, f_idx, M, F) -> np.ndarray:
    """Rows of the full plan's output that the sample operator's rows are, in its order."""
    return np.array([(w * M + m) * F + f for w in w_idx for m in m_idx for f in f_idx])


def _init(cfg, n_planes):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    op, *_ = sample_operator(cfg, n_planes)
    _STATE["op"] = op


def _adjoint_part(args):
    """Adjoint of the sample restricted to the (wave, mix) blocks `blocks` (linear in the blocks)."""
    from oracle import adjoint_quick_cpu
    blocks, u = args
    op = _STATE["op"]
    n_f = len(op.measurements[0].mixes[0].f_idx)
    meas, rows = [], []
    for w, meas_w in enumerate(op.measurements):
        keep = [m for m in range(len(meas_w.mixes)) if (w, m) in blocks]
        meas.append(dataclasses.replace(meas_w, mixes=[meas_w.mixes[m] for m in keep]))
        M = len(meas_w.mixes)
        for m in keep:
            rows.extend(range((w * M + m) * n_f, (w * M + m + 1) * n_f))
    sub = dataclasses.replace(op, measurements=meas)
    return adjoint_quick_cpu(sub, u[np.array(rows, dtype=int)])


def adjoint_parallel(cfg, n_planes, op, u, processes=None) -> np.ndarray:
    """adjoint_quick_cpu(op, u) summed over (wave, mix) blocks computed in a spawn pool."""
    blocks = [(w, m) for w in range(len(op.measurements)) for m in range(len(op.measurements[w].mixes))]
    n = max(1, min(len(blocks), processes or (os.cpu_count() or 1)))
    chunks = [set(blocks[i::n]) for i in range(n)]
    with mp.get_context("spawn").Pool(n, initializer=_init, initargs=(cfg, n_planes)) as pool:
        parts = pool.map(_adjoint_part, [(c, u) for c in chunks])
    return np.sum(parts, axis=0)
