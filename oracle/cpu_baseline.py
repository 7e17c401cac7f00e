"""Timed CPU baseline: the FP64 oracle operator on a bounded sample of a workload.

TEST/BENCH INFRASTRUCTURE ONLY: used by ``bench.py``'s ``cpu_baseline`` leg
(timed, and to check the device path on the sample's rows) and by
``bench.py --impl reference``.  The reference's own CPU operator
(MATLAB ``forward_quick_cpu`` / ``adjoint_quick_cpu``) cannot run on these
machines; its restatement in :mod:`oracle.born_oracle` keeps the same loop
structure (per measurement, mix and active element: gather the shifted
transfer function, form Phi = h .* p_in .* pref, multiply with BLAS), and
that is what is timed here.

The sample keeps the full grid and every element but only ``n_waves`` waves
and ``n_freq`` frequencies; the work of the operator is linear in
(waves x frequencies), so the full-workload rate is the sample rate divided
by ``(S_full / S_sample)``.  Mixes are split over a ``spawn`` process pool,
one worker per host core; each worker builds the sample's tables itself
(untimed) and the timed region covers the forward and adjoint applies.
"""

from __future__ import annotations

import multiprocessing as mp
import os
import time

import numpy as np

_STATE = {}


def _sample_config(name: str, n_waves: int, n_freq: int, n_planes=None):
    """The workload restricted to n_waves waves, n_freq frequencies and (optionally) the first
    n_planes axial grid planes; every grid point costs the same work, so the planes scale
    linearly."""
    import dataclasses
    from oracle import configs
    cfg = configs.config(name)
    f_idx = np.linspace(0, len(cfg.f) - 1, n_freq).round().astype(int)
    cfg.band = (float(cfg.f.min()), float(cfg.f.max()))  # the full workload's excitation spectrum
    cfg.f = cfg.f[f_idx]
    cfg.waves = cfg.waves[:n_waves]
    if n_planes is not None:
        axes = tuple(cfg.setup.n_points_axis)
        cfg.setup = dataclasses.replace(cfg.setup, n_points_axis=axes[:-1] + (min(n_planes, axes[-1]),))
    return cfg


def _init(name, n_waves, n_freq, seed, n_objects=1, n_planes=None):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import configs
    cfg = _sample_config(name, n_waves, n_freq, n_planes)
    b = configs.build(cfg)
    rng = np.random.default_rng(seed)
    P = cfg.setup.n_points
    gamma = rng.standard_normal((P, n_objects))
    _STATE.update(b=b, gamma=gamma)


def _work(args):
    """Forward and adjoint restricted to a chunk of mixes of every measurement.  With ``want``
    the chunk's forward rows and the first column of its adjoint come back too (for checking a
    device result against them; they are computed inside the timed region anyway)."""
    import dataclasses
    from oracle import adjoint_quick_cpu, forward_quick_cpu
    lo, hi = args[0], args[1]
    want = len(args) > 2 and args[2]
    if hi <= lo:  # warm-up call: the initializer has built the tables
        return 0.0, 0.0, None, None
    b = _STATE["b"]
    meas = [dataclasses.replace(m, mixes=m.mixes[lo:hi]) for m in b.op.measurements]
    op = dataclasses.replace(b.op, measurements=meas)
    t0 = time.perf_counter()
    u = forward_quick_cpu(op, _STATE["gamma"])
    g = adjoint_quick_cpu(op, u)
    t = time.perf_counter() - t0
    return t, float(np.abs(g).sum()), (u if want else None), (g[:, 0].copy() if want else None)


def time_sample(name: str = "c1", n_waves: int = 1, n_freq: int = 8, processes: int | None = None,
                repeats: int = 1, seed: int = 0, n_objects: int = 1, n_mixes: int | None = None,
                n_planes: int | None = None, check: bool = False):
    """Seconds per forward+adjoint apply of the full workload, extrapolated from a sample.

    With ``check`` the result also holds the sample's FP64 outputs (``"check"``): the forward rows
    of wave 0 (mix-major, then the sample frequencies ``f_idx`` of the full workload), the first
    column of the adjoint of those rows, the seed of the real Gaussian gamma (P_sample x
    n_objects) and the sizes, for comparing a device apply of the full workload with them.

    ``n_mixes`` keeps only the first receive mixes of every wave (work is linear
    in the mixes when every mix has the same active elements, as in the
    benchmark workloads); ``n_planes`` keeps only the first axial grid planes
    (work is linear in the grid points).  Returns a dict with the sample description, the
    measured seconds and the extrapolated full-workload applies/s.
    """
    from oracle import configs
    full = configs.config(name)
    S_full = len(full.waves) * len(full.f)
    S_sample = n_waves * n_freq
    P_full = full.setup.n_points
    P_sample = _sample_config(name, n_waves, n_freq, n_planes).setup.n_points
    n_mix_full = full.setup.n_elements if full.mixing == "identity" else full.n_mixes
    n_mix = min(n_mix_full, n_mixes or n_mix_full)
    procs = processes or os.cpu_count() or 1
    procs = max(1, min(procs, n_mix))
    bounds = np.linspace(0, n_mix, procs + 1).round().astype(int)
    chunks = [(int(bounds[i]), int(bounds[i + 1])) for i in range(procs)]
    # one BLAS thread per worker: the spawned interpreters read these before importing numpy
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs, initializer=_init, initargs=(name, n_waves, n_freq, seed, n_objects, n_planes)) as pool:
        pool.map(_work, [(0, 0)] * procs)  # wait until every worker holds its tables
        times = []
        outs = None
        for r in range(repeats):
            # critical path of the parallel apply: the slowest worker's own compute time
            res = pool.map(_work, [(lo, hi, check and r == 0) for lo, hi in chunks], chunksize=1)
            times.append(max(t for t, _, _, _ in res))
            if check and r == 0:
                outs = res
    t_sample = min(times)
    scale = (S_full / S_sample) * (n_mix_full / n_mix) * (P_full / P_sample)
    t_full = t_sample * scale
    result = {
        "seconds_sample": t_sample,
        "seconds_per_repeat": times,
        "scale": scale,
        "seconds_full_apply": t_full,
        "applies_per_s": n_objects / t_full,  # object-applies: all columns go through one BLAS call per element
        "cores": procs,
        "sample": f"{n_waves} of {len(full.waves)} waves x {n_freq} of {len(full.f)} frequencies x {n_objects} "
                  f"gamma columns, "
                  + (f"full {'x'.join(map(str, full.setup.n_points_axis))} grid"
                     if P_sample == P_full else f"{P_sample} of {P_full} grid points (the first {n_planes} axial planes)")
                  + f", all {full.setup.n_elements} elements; "
                  f"one forward + one adjoint (FP64 numpy/scipy restatement of forward_quick_cpu/adjoint_quick_cpu), "
                  f"{n_mix} of {n_mix_full} receive mixes split over {procs} spawn processes; full-workload rate = "
                  f"sample rate x {S_sample}/{S_full} x {n_mix}/{n_mix_full}"
                  + (f" x {P_sample}/{P_full}" if P_sample != P_full else ""),
    }
    if check:
        f_idx = np.linspace(0, len(full.f) - 1, n_freq).round().astype(int)
        result["check"] = {"u_rows": np.concatenate([o[2] for o in outs], axis=0),
                           "g0": np.sum([o[3] for o in outs], axis=0), "f_idx": [int(i) for i in f_idx],
                           "n_mix": n_mix, "P_sample": P_sample, "seed": seed}
    return result


if __name__ == "__main__":
    import json
    print(json.dumps(time_sample()))
