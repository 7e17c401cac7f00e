"""Frequency-split FP64 oracle for problems of the uneven-batch solver loop (test/bench infrastructure).

TEST/BENCH INFRASTRUCTURE ONLY: used by ``tests/`` to check the device LASSO iterations
(``cui_born_lasso``) on problems of the uneven batch, and by ``bench.py``'s ``cpu_baseline`` leg of
that workload.  Nothing in the product imports it.

The Born operator is block-diagonal in frequency: row (w, m, f) of the forward
(``operator_born.m:332-452``) depends on the tables at frequency f only, and the adjoint
(``operator_born.m:456-596``) is the sum over frequencies of each frequency's block.  Each
``spawn`` worker builds the oracle operator restricted to a subset of the frequencies (keeping
the full band's excitation spectrum, so its rows are rows of the whole operator).  A forward is
the union of the workers' rows, written where row (w, m, f) of the whole operator sits, at
``(w * M + m) * F + f``.  An adjoint is the sum of the workers' partial gradients.  The
proximal-gradient iterations then run in the parent through :func:`oracle.solvers.lasso_ista`,
unchanged.
"""

from __future__ import annotations

import dataclasses
import multiprocessing as mp
import os

import numpy as np


def _worker(conn, cfg, f_idx):
    from oracle import adjoint_quick_cpu, configs, forward_quick_cpu
    sub = dataclasses.replace(cfg)
    sub.band = (float(np.min(cfg.f)), float(np.max(cfg.f))) if cfg.band is None else cfg.band
    sub.f = np.asarray(cfg.f)[f_idx]
    op = configs.build(sub).op
    conn.send(("ready", len(op.measurements[0].mixes)))
    while True:
        cmd, x = conn.recv()
        if cmd == "forward":
            conn.send(forward_quick_cpu(op, x))
        elif cmd == "adjoint":
            conn.send(adjoint_quick_cpu(op, x))
        else:
            conn.close()
            return


class FrequencySplitOracle:
    """The oracle operator of ``cfg`` (an ``oracle.configs.BornConfig``) over ``processes``
    spawn workers, each holding a contiguous subset of the frequencies.  Use as a context
    manager, or call :meth:`close`."""

    def __init__(self, cfg, processes: int | None = None):
        F = len(cfg.f)
        n = max(1, min(F, processes or os.cpu_count() or 1))
        bounds = np.linspace(0, F, n + 1).round().astype(int)
        self.f_sets = [np.arange(bounds[i], bounds[i + 1]) for i in range(n) if bounds[i + 1] > bounds[i]]
        self.F, self.W = F, len(cfg.waves)
        self.P = cfg.setup.n_points
        ctx = mp.get_context("spawn")
        self._conns, self._procs = [], []
        # one BLAS thread per worker: a spawned interpreter reads these before it imports numpy
        saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        os.environ.update({v: "1" for v in saved})
        try:
            for fs in self.f_sets:
                a, b = ctx.Pipe()
                p = ctx.Process(target=_worker, args=(b, cfg, fs), daemon=True)
                p.start()
                self._conns.append(a)
                self._procs.append(p)
        finally:
            for v, old in saved.items():
                if old is None:
                    os.environ.pop(v, None)
                else:
                    os.environ[v] = old
        self.M = None
        for c in self._conns:
            tag, M = c.recv()
            self.M = M
        WM = self.W * self.M
        # rows of the whole operator that each worker's rows are, in the worker's order
        self.rows = [np.array([wm * F + f for wm in range(WM) for f in fs]) for fs in self.f_sets]
        self.n_observations = WM * F

    def forward(self, gamma: np.ndarray) -> np.ndarray:
        g = np.asarray(gamma, dtype=np.complex128)
        for c in self._conns:
            c.send(("forward", g))
        out = np.zeros((self.n_observations,) + g.shape[1:], dtype=np.complex128)
        for c, rows in zip(self._conns, self.rows):
            out[rows] = c.recv()
        return out

    def adjoint(self, u: np.ndarray) -> np.ndarray:
        u = np.asarray(u, dtype=np.complex128)
        for c, rows in zip(self._conns, self.rows):
            c.send(("adjoint", u[rows]))
        return np.sum([c.recv() for c in self._conns], axis=0)

    def lasso(self, u, lam, step: float, n_iter: int):
        """``oracle.solvers.lasso_ista`` with this split operator: ``(gamma, loss)``."""
        from oracle.solvers import lasso_ista
        return lasso_ista(None, u, lam, step, n_iter, forward=self.forward, adjoint=self.adjoint,
                          n_points=self.P)

    def close(self):
        for c in self._conns:
            try:
                c.send(("stop", None))
            except (BrokenPipeError, OSError):
                pass
        for p in self._procs:
            p.join(timeout=30)
        self._conns, self._procs = [], []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def lasso_problem_config(side: int, n_elements: int, f, angles_deg, density: float = 0.02, seed: int = 0,
                         name: str = "lasso"):
    """BornConfig of one problem of the uneven batch: a side x side lossless 2D grid at the
    linear-array pitch, ``n_elements`` elements, quasi-plane waves at ``angles_deg``."""
    from oracle import configs
    s = configs._setup_2d(side, side, n_elements, configs.LOSSLESS)
    return configs.BornConfig(name, s, np.asarray(f, dtype=float), [configs.Wave("qpw", (float(a),)) for a in angles_deg],
                              density=density, seed=seed)
