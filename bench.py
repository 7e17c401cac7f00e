"""Benchmark of the GB300 Born operator: forward + adjoint applies per second.

Workload (default ``2d-batched``, the batched split-precision configuration):
2D, 512x512 FOV at 76.2 um, 128-element linear array, 16 random-apodization
incident waves mixed into 32 receive signals by +-1 weights, 128 frequencies
over 2.5-5.5 MHz, 64 right-hand-side gamma columns.  One step = one gradient
of 0.5||Phi gamma - u||^2 (forward, residual, adjoint) for all 64 columns
through the C-ABI (``cui_born_vjp``) -- 64 forward + adjoint applies.  The
same plan then times the plain FP32 path on the same inputs, so the line
carries the split-BF16 / FP32 speed-up and the split-BF16 gradient's error
against the FP32 one.  ``--workload 2d-gradient`` runs the single-object
configuration (11 quasi-plane waves, 192 frequencies, time-causal medium).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Prints one JSON line.  ``value`` is applies/s over all ranks with inputs
resident in HBM; ``e2e`` is the same metric through the host (FP64, MEX
semantics) entry point, with host<->device copies inside the timed region.
``--impl reference`` times the reference's CPU operator (its FP64
restatement) on the host cores instead.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Born fwd+adj applies/s, % roofline; batched split-BF16 vs FP32 at rel err≤1e-5"
ORACLE_NAME = {"2d-plain": "c0", "2d-gradient": "c1", "2d-batched": "c2", "3d": "c3"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="2d-batched")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-greedy", action="store_true",
                    help="single-object workloads: skip timing the device OMP and CoSaMP solvers")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--fp32-steps", type=int, default=3,
                    help="steps of the plain FP32 path timed after the main region (0: skip)")
    ap.add_argument("--precision", choices=["fp32", "bf16x3", "bf16x3-folded", "auto"], default=None,
                    help="contraction path: FP32 CUDA cores, split-BF16 tcgen05 tensor cores over slots and "
                         "elements, split-BF16 tcgen05 GEMMs against the folded operator stored in device memory, "
                         "or the per-plan autotuner (default: bf16x3-folded for 2d-batched, fp32 for 3d, auto "
                         "otherwise)")
    ap.add_argument("--table-storage", choices=["auto", "stored", "streamed", "generated"], default=None,
                    help="lateral transfer-function table: stored once; regenerated every apply in chunks of "
                         "frequencies (streamed, 3D); or generated inside the contraction kernels where they use "
                         "it (3D); auto stores it unless it does not fit in device memory (default: streamed for "
                         "3d, whose configuration recomputes the table; auto otherwise)")
    ap.add_argument("--lasso-streams", type=int, default=4,
                    help="2d-lasso: concurrent streams the problems are spread over inside the graph")
    ap.add_argument("--lasso-problems", type=int, default=256,
                    help="2d-lasso: how many of the seeded uneven problems the job holds (the configuration's 256)")
    ap.add_argument("--lasso-budget-gb", type=float, default=None,
                    help="2d-lasso: device memory the plans of one batch may hold (default: 85 %% of free memory)")
    ap.add_argument("--lasso-iters", type=int, default=50)
    ap.add_argument("--n-freq", type=int, default=None,
                    help="keep only the first N frequencies (reduced case for profiler captures)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---- replicas (one process per GPU; the path needs no data exchange for this metric) --------
def replicas_begin(world: int, backend: str = "nccl"):
    """Process group of the replicas (torchrun's env:// rendezvous); None for one process."""
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend)
    return dist


def replicas_barrier(dist):
    if dist is not None:
        dist.barrier()


def replicas_max_ms(dist, ms: float, device=None) -> float:
    """The slowest replica's timed region: every replica waits for it, so it is the job's time."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_replica: float, ms: float) -> float:
    """Units all replicas processed per second of the slowest replica's time (weak scaling)."""
    return world * units_per_replica / (ms / 1e3)


def replicas_end(dist):
    if dist is not None:
        dist.destroy_process_group()


def relaunch_as_replicas(n: int) -> int:
    """``--gpus N`` outside torchrun: run this command as N replica processes under
    torch.distributed.run (rendezvous on 127.0.0.1) and return its exit code."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", os.environ.get("MASTER_PORT", "29511"),
           str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def peaks():
    """Roofline denominators: the measured copy bandwidth and cuBLAS bf16 rate (MEASURED_PEAKS.json), else the fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0, "source": "fallback"}


def launch_traffic(workload: str, kernel: str, n_freq: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (scaled by frequencies), or None."""
    tf = ROOT / "profiles" / "traffic.json"
    if not tf.exists():
        return None
    rec = json.loads(tf.read_text()).get(f"{workload}:{kernel}")
    if not rec:
        return None
    return rec["bytes_per_frequency"] * n_freq


def time_greedy(op):
    """Wall-clock time of the device greedy solvers on one measured column of this plan:
    OMP (cui_born_omp, 32 atoms) and CoSaMP (cui_born_cosamp, sparsity 16, 8 iterations), on
    data from 16 seeded point scatterers.  Both are host-driven loops that read one residual
    norm per iteration; one adjoint apply of a single column is timed beside them."""
    import numpy as np
    import torch
    rng = np.random.default_rng(77)
    P = op.n_points
    g = np.zeros((P, 1), dtype=np.complex64)
    idx = rng.choice(P, 16, replace=False)
    g[idx, 0] = (1.0 + rng.random(16)) * np.exp(2j * np.pi * rng.random(16))
    y = op.forward(torch.from_numpy(g).cuda())[:, 0].contiguous()
    op.omp(y, 2)
    op.cosamp(y, 4, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    atoms, _, rel = op.omp(y, 32)
    t_omp = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, _, rel_c = op.cosamp(y, 16, 8)
    t_cos = time.perf_counter() - t0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    yy = y[:, None]
    op.adjoint(yy)
    e0.record(torch.cuda.current_stream())
    for _ in range(5):
        op.adjoint(yy)
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    return {"omp": {"atoms": int(len(atoms)), "ms": 1e3 * t_omp, "ms_per_atom": 1e3 * t_omp / max(1, len(atoms)),
                    "rel_residual": float(rel[-1])},
            "cosamp": {"sparsity": 16, "iterations": int(len(rel_c)), "ms": 1e3 * t_cos,
                       "ms_per_iteration": 1e3 * t_cos / max(1, len(rel_c)), "rel_residual": float(rel_c[-1])},
            "adjoint_one_column_ms": e0.elapsed_time(e1) / 5,
            "data": "16 seeded point scatterers, noiseless"}


def occupancy_sweep(op, densities=(0.001, 0.005, 0.02, 0.05, 0.0625, 0.1, 0.25, 1.0)):
    """FP32 forward of one column against the density of gamma's nonzeros.

    The reference's forward contracts only the occupied grid points (``operator_born.m:361``,
    ``combined_quick_gpu.cu:457-499``).  The plan lists them on the device and takes the
    compacted contraction at up to N_points/16 of them (N_points/32 when the table is streamed or
    generated), otherwise the dense kernels.  For each
    density (seeded positions, N(0,1) values) this times 10 forwards with CUDA events, notes the
    path, and checks the result against the dense kernels on the same gamma (occupancy limit 0).
    """
    import numpy as np
    import torch
    prev = op.precision
    op.set_precision("fp32")
    P = op.n_points
    limit = P // (16 if op.table_storage == "stored" else 32)  # the plan's default limit
    rng = np.random.default_rng(5)
    rows = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for d in densities:
        nnz = max(1, int(round(d * P)))
        g = np.zeros((P, 1), dtype=np.complex64)
        g[rng.choice(P, nnz, replace=False), 0] = rng.standard_normal(nnz)
        gt = torch.from_numpy(g).cuda()
        op.set_occupancy_limit(-1)
        for _ in range(2):
            u = op.forward(gt)
        torch.cuda.synchronize()
        e0.record(torch.cuda.current_stream())
        for _ in range(10):
            u = op.forward(gt)
        e1.record(torch.cuda.current_stream())
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        op.set_occupancy_limit(0)
        u_dense = op.forward(gt)
        op.set_occupancy_limit(-1)
        rows.append({"density": d, "nnz": nnz, "forward_ms": ms,
                     "path": "compacted" if nnz <= limit else "dense",
                     "rel_l2_vs_dense": float((u - u_dense).norm() / u_dense.norm())})
    op.set_precision(prev)
    return {"rows": rows, "threshold_points": limit,
            "what": "FP32 forward of one seeded gamma column per density: ms per forward (CUDA events, 10 "
                    "forwards), the path taken, and the relative L2 difference from the dense kernels"}


def roofline_of(args, info, kt, B, clk, p_used: float = 1.0):
    """Roofline of the dominant contraction kernel of one apply.

    Algorithmic work (the channel-contraction work count): E = sum over slots of min(rows of the slot,
    distinct active elements) x P_used complex multiply-adds per object (``channel_macs``:
    the element sum folded into the receive mixes; P_used = the union occupancy of the
    forward's gamma columns, all points for the adjoint), x B objects.

    Split-BF16 (tensor cores): 24 FLOP per complex MAC (4 real products x 3 bf16 products
    x 2) against the measured bf16 tensor peak.  The folded-operator GEMMs stream the
    stored matrix (8 B per entry and launch) at 192 FLOP per byte, below the ridge point
    (peak FLOP/s / peak B/s), so their governing roof is HBM: ``bound`` "hbm" with the
    bytes one launch must move (matrix + operands + outputs) and the tensor figure beside.
    FP32 (CUDA cores): 8 FLOP per complex MAC against 152 SMs x 128 lanes x 2 x the sampled
    SM clock.  ``executed_*`` counts the multiply-adds the kernel actually performs (the
    element contraction: S x E x P, all points).
    """
    pk = peaks()
    dom = "forward" if kt["ms_forward"] >= kt["ms_adjoint"] else "adjoint"
    t_launch = kt["ms_" + dom] / max(1, kt["n_" + dom]) / 1e3
    P = info["n_points"]
    folded = args.precision == "bf16x3-folded"
    alg_macs = info["channel_macs"] * B * (p_used if dom == "forward" else 1.0)
    exec_macs = (info["channel_macs"] if folded else info["contraction_macs"]) * B
    # table bytes one launch moves: a stored table is read once; a streamed one is written by the chunk
    # generator and read back (the full table, chunk by chunk); a generated one never leaves the SMs
    table = {"stored": info["table_bytes"], "streamed": 2 * args.full_table_bytes, "generated": 0}[args.table_used]
    if folded:
        compulsory = info["folded_bytes"] + 8 * B * P + 8 * B * info["n_observations"]
    else:
        compulsory = table + info["incident_bytes"] + 8 * B * P + 8 * B * info["n_observations"]
    tc = args.precision != "fp32"
    # every 2D benchmark workload (4 grid points per pitch, lines a multiple of 8) runs the line-unit kernels;
    # 3D setups run the FP32 kernels under register ceilings (dense3) or with the generator inside (gen)
    fp32_kind = "dense" if args.n_dims == 2 else ("gen" if args.table_used == "generated" else "dense3")
    kernel = {("forward", True): "fwd_tc2_kernel", ("adjoint", True): "adj_tc2_kernel",
              ("forward", False): f"fwd_{fp32_kind}_kernel", ("adjoint", False): f"adj_{fp32_kind}_kernel"}[(dom, tc)]
    if folded:
        kernel = "phi_gemm_kernel<" + ("true" if dom == "adjoint" else "false") + ">"
    traffic = launch_traffic(args.workload, kernel, args.n_freq_used)
    hbm = {"compulsory_bytes": compulsory, "achieved_gbs": compulsory / t_launch / 1e9,
           "peak_gbs": pk["hbm_gbs"], "frac": compulsory / t_launch / 1e9 / pk["hbm_gbs"],
           "traffic_over_compulsory": (traffic / compulsory) if traffic else None}
    # the reference writes Phi (8 B per complex entry) and reads it back through cublasCgemm: the
    # rate at which this launch covers those bytes, against the HBM peak (the plain-FP32 criterion)
    hbm["phi_equivalent_gbs"] = 8.0 * alg_macs / t_launch / 1e9
    hbm["phi_equivalent_frac"] = hbm["phi_equivalent_gbs"] / pk["hbm_gbs"]
    sm_mhz = clk.get("sm_mhz") or pk["sm_max_mhz"]
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    launch_ms = {"forward": kt["ms_forward"] / max(1, kt["n_forward"]),
                 "adjoint": kt["ms_adjoint"] / max(1, kt["n_adjoint"])}
    work = {"algorithmic_complex_macs_per_launch": alg_macs, "executed_complex_macs_per_launch": exec_macs,
            "p_used_fraction": p_used if dom == "forward" else 1.0,
            "definition": "E = sum over slots of min(rows, distinct active elements) x P_used per object "
                          "(channel_macs), x objects; P_used = union occupancy of the forward's gamma"}
    peak_src = (f"{pk['source']} bf16 burst (MEASURED_PEAKS.json bf16_tflops)" if pk["source"] == "measured"
                else "fallback")
    if tc:
        flops = 24.0 * alg_macs
        achieved = flops / t_launch / 1e12
        tensor = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                  "frac": achieved / pk["bf16_tflops"], "peak_source": peak_src,
                  "executed_tflops": 24.0 * exec_macs / t_launch / 1e12,
                  "achieved_definition": "24 FLOP per complex MAC (4 real x 3 split-BF16 products x 2) x the "
                                         "algorithmic complex MACs per launch / average launch time"}
        if folded:
            return {"bound": "hbm", "achieved": hbm["achieved_gbs"], "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "frac": hbm["frac"], "traffic": traffic, "kernel": kernel,
                    "peak_source": "measured HBM copy (MEASURED_PEAKS.json hbm_gbs)" if pk["source"] == "measured"
                    else "fallback",
                    "achieved_definition": "bytes one launch must move (folded matrix, 8 B per observation x point, "
                                           "+ gamma and observations in FP32) / average launch time; the GEMM runs "
                                           "at 192 FLOP/B, below the bf16 ridge point, so HBM governs",
                    "tensor": tensor, "work": work, "hbm": hbm, "launch_ms": launch_ms}
        return dict(tensor, traffic=traffic, kernel=kernel, work=work, hbm=hbm, launch_ms=launch_ms,
                    flops_per_launch=flops)
    flops = 8.0 * alg_macs
    achieved = flops / t_launch / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": achieved / fp32_peak, "traffic": traffic, "kernel": kernel,
            "peak_source": "152 SMs x 128 FP32 lanes x 2 FLOP x median sampled SM clock",
            "achieved_definition": "8 FLOP per complex MAC x the algorithmic complex MACs per launch / average "
                                   "launch time",
            "executed_tflops": 8.0 * exec_macs / t_launch / 1e12,
            "flops_per_launch": flops, "work": work, "hbm": hbm, "launch_ms": launch_ms}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None
        self.t0 = self.t1 = None

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        import datetime
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                if self.t0 is not None and not (self.t0 - 0.25 <= ts <= (self.t1 or ts) + 0.25):
                    continue
                sm.append(float(r[2]))
                smax = float(r[3])
            except ValueError:
                continue
            for n, v in zip(names, r[6:10]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# bounded CPU samples (about 10-30 s of host work): (waves, frequencies, receive mixes or None = all,
# axial planes or None = all); "cores" = one receive mix per host core (the 32 mixes of 2d-batched)
CPU_SAMPLE = {"2d-plain": (1, 64, None, None), "2d-gradient": (1, 96, None, None), "2d-batched": (1, 1, "cores", None),
              "3d": (1, 2, None, None)}
# per-step samples of the reference arm, small enough for --steps K --warmup W to end within minutes
REF_SAMPLE = {"2d-plain": (1, 2, None, None), "2d-gradient": (1, 1, None, 128), "2d-batched": (1, 1, "cores", 128),
              "3d": (1, 1, None, 2)}


def sample_mixes(nm):
    return min(32, max(8, os.cpu_count() or 8)) if nm == "cores" else nm


def cpu_baseline(workload: str, n_objects: int, op=None, w=None):
    """Times the FP64 oracle on the workload's bounded sample.  With the device plan ``op`` of the
    full workload ``w`` it also checks the plan's current path against the sample's FP64 outputs
    (returned as ``check``): the forward rows of wave 0 at the sample's frequencies and receive
    mixes, for the sample's seeded real Gaussian gamma (zero outside the sample's grid planes), and
    the first column of the adjoint of exactly those rows."""
    from oracle.cpu_baseline import time_sample
    nw, nf, nm, npl = CPU_SAMPLE[workload]
    r = time_sample(ORACLE_NAME[workload], n_waves=nw, n_freq=nf, n_objects=n_objects, n_mixes=sample_mixes(nm),
                    n_planes=npl, check=op is not None)
    out = {"value": r["applies_per_s"], "unit": "applies/s", "cores": r["cores"], "kind": "port",
           "sample": r["sample"], "seconds_sample": r["seconds_sample"]}
    check = None
    if op is not None:
        import numpy as np
        import torch
        c = r["check"]
        F, Ps = len(w.f), c["P_sample"]
        gam = np.zeros((op.n_points, n_objects), dtype=np.complex64)
        gam[:Ps] = np.random.default_rng(c["seed"]).standard_normal((Ps, n_objects))
        rows = np.array([m * F + fi for m in range(c["n_mix"]) for fi in c["f_idx"]])
        u_dev = op.forward(torch.from_numpy(gam).cuda()).cpu().numpy().astype(np.complex128)[rows]
        u_in = np.zeros((op.n_observations, n_objects), dtype=np.complex64)
        u_in[rows] = c["u_rows"]
        g_dev = op.adjoint(torch.from_numpy(u_in).cuda()).cpu().numpy().astype(np.complex128)[:Ps, 0]
        rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
        check = {"rel_l2_forward": rel(u_dev, c["u_rows"]), "rel_l2_adjoint": rel(g_dev, c["g0"]),
                 "rows": int(len(rows)), "columns": int(n_objects),
                 "what": "device path vs the FP64 oracle on the CPU sample: forward rows of wave 0 at the sample's "
                         "frequencies and mixes (all columns), adjoint of those rows (first column)"}
    return out, check


TABLE_STORAGE = {
    "stored": "stored: built on the device once per plan, read every apply",
    "streamed": "streamed: regenerated on the device every apply, one chunk of frequencies at a time into a "
                "chunk buffer, then read by the contraction kernels (never stored whole)",
    "generated": "generated: computed inside the contraction kernels where each entry is staged (never stored)",
}


def full_table_bytes(w) -> int:
    """Bytes of the stored lateral table [F][Nz][Noy][Nox] (FP32 complex) of a workload."""
    nl = len(w.n_points_axis) - 1
    n = len(w.f) * w.n_points_axis[-1]
    for a in range(nl):
        ppp = int(round(w.pitch_axis[a] / w.delta_axis[a]))
        n *= w.n_points_axis[a] + (w.n_elements_axis[a] - 1) * ppp
    return 8 * n


def workload_config(w, B):
    return {"workload": f"{w.name}: {'x'.join(map(str, w.n_points_axis))} FOV, {len(w.f)} frequencies, "
                        f"{w.n_elements} elements, {len(w.waves)} waves, {w.absorption['kind']} medium; "
                        f"one step = VJP of 0.5||Phi g - u||^2 (forward + adjoint)",
            "n_points": w.n_points, "n_frequencies": len(w.f), "n_waves": len(w.waves),
            "n_elements": w.n_elements, "n_objects": B,
            "l2": "inputs larger than L2 (incident fields and transfer-function table, several GB, re-read every step)"}


def run_reference(args):
    """The reference's CPU operator (its FP64 restatement, the oracle port) on the host cores.

    Every step times one forward + adjoint over a bounded sample of the workload (``REF_SAMPLE``,
    split over one spawn process per host core); ``warmup`` + ``steps`` such samples run and
    ``ms_per_step`` is the median sample step as measured.  ``value`` scales that step to the
    full workload (linear in waves x frequencies x mixes x grid points): the line says so with
    ``extrapolated`` and ``scale_factor``.
    """
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from comp_ui_toolbox_gb300.workloads import workload
    w = workload(args.workload if args.workload in ORACLE_NAME else "2d-gradient")
    B = w.n_objects if args.workload == "2d-batched" else 1
    from oracle.cpu_baseline import time_sample
    nw, nf, nm, npl = REF_SAMPLE[w.name]
    t0 = time.perf_counter()
    r = time_sample(ORACLE_NAME[w.name], n_waves=nw, n_freq=nf, n_objects=B, n_mixes=sample_mixes(nm),
                    n_planes=npl, repeats=args.warmup + args.steps)
    wall = time.perf_counter() - t0
    timed = sorted(r["seconds_per_repeat"][args.warmup:])
    t_step = timed[len(timed) // 2]
    value = B / (t_step * r["scale"])
    line = {"metric": METRIC, "value": value, "unit": "applies/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": workload_config(w, B),
            "impl": "reference",
            "extrapolated": True, "scale_factor": r["scale"],
            "step_definition": "one forward + adjoint of the bounded sample below (ms_per_step as measured, median "
                               "of the timed steps); value = objects / (sample step seconds x scale_factor)",
            "wall_s": wall,
            "cpu_baseline": {"value": value, "unit": "applies/s", "cores": r["cores"], "kind": "port",
                             "host_cores": os.cpu_count(), "sample": r["sample"]},
            "e2e": {"value": value, "unit": "applies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_env()
    dist = replicas_begin(world)
    torch.cuda.set_device(local)
    from comp_ui_toolbox_gb300 import OperatorBorn, launch_count
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload(args.workload)
    if args.n_freq:
        w.f = w.f[: args.n_freq]
    args.n_freq_used = len(w.f)
    B = w.n_objects if args.workload == "2d-batched" else 1
    t0 = time.perf_counter()
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=local, max_objects=B, table_storage=args.table_storage)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    args.table_used = op.table_storage
    args.n_dims = len(w.n_points_axis)
    args.full_table_bytes = full_table_bytes(w)
    P, N = op.n_points, op.n_observations

    # data: u = Phi gamma_true + noise (20 dB for 2d-plain, 30 dB otherwise).  The step is the VJP at
    # the workload's own configured gamma: further seeded columns of its sparsity (2d-plain 2 %,
    # 2d-batched 64 columns at 3 %, 3d 1 %), or a seeded Gaussian gamma for 2d-gradient, whose
    # configuration takes the gradient there
    gamma_true = torch.from_numpy(w.gamma(n_objects=B).astype(np.complex64)).cuda()
    u_clean = op.forward(gamma_true)
    gen = torch.Generator(device="cuda").manual_seed(7)
    noise = torch.randn(u_clean.shape, dtype=torch.complex64, device="cuda", generator=gen)
    snr_db = 20.0 if args.workload == "2d-plain" else 30.0
    snr = 10 ** (-snr_db / 20)
    u_meas = (u_clean + noise * (u_clean.abs().pow(2).mean().sqrt() / noise.abs().pow(2).mean().sqrt()) * snr).contiguous()
    if args.workload != "2d-gradient":
        gamma = torch.from_numpy(w.gamma(seed=w.seed + 1, n_objects=B).astype(np.complex64)).cuda()
        gamma_kind = f"{B} column(s) at {w.density:.0%} Gaussian sparsity (seeded)"
    else:
        gamma = torch.randn((P, B), dtype=torch.float32, device="cuda", generator=gen).to(torch.complex64)
        gamma_kind = "seeded Gaussian (dense)"
    # column-major storage (each column contiguous, the layout of MATLAB arrays and of the C-ABI), so
    # that the Python wrapper hands the columns to the library without a transposing copy
    gamma = gamma.t().contiguous().t()
    u_meas = u_meas.t().contiguous().t()
    # union occupancy of the forward's columns: the reference's forward contracts only these points
    p_used = float((gamma.abs().amax(dim=1) > 0).float().mean())
    autotune = None
    if args.precision == "auto":  # the per-plan autotuner keeps the faster path; the bench then runs that
        autotune = op.autotune(B)
        args.precision = autotune["precision"]
    accuracy = None
    t_fold = None
    if args.precision != "fp32":
        # same plan, both precisions: relative L2 of the split-BF16 gradient against the FP32 one
        op.set_precision("fp32")
        g32, _ = op.vjp(gamma, u_meas)
        t0 = time.perf_counter()
        op.set_precision(args.precision)
        torch.cuda.synchronize()
        if args.precision == "bf16x3-folded":
            t_fold = time.perf_counter() - t0
        op.refresh_info()
        gtc, _ = op.vjp(gamma, u_meas)
        accuracy = {"rel_l2_grad_vs_fp32": float((gtc - g32).norm() / g32.norm()),
                    "note": "the FP32 path itself is <= 2e-7 from the FP64 oracle on the test workloads"}
        del g32, gtc

    def step():
        return op.vjp(gamma, u_meas)

    with ClockSampler(local) as clocks:
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        replicas_barrier(dist)
        stream = torch.cuda.current_stream()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        op.timing(True)
        op.timing()  # clear
        n0 = launch_count()
        torch.cuda.synchronize()
        clocks.mark_start()
        ev0.record(stream)
        for _ in range(args.steps):
            grad, loss = step()
        ev1.record(stream)
        torch.cuda.synchronize()
        clocks.mark_end()
    replicas_barrier(dist)
    launches = launch_count() - n0
    kt = op.timing()
    op.timing(False)
    ms = replicas_max_ms(dist, ev0.elapsed_time(ev1), device="cuda")
    ms_step = ms / args.steps
    value = whole_job_rate(world, args.steps * B, ms)

    # end to end through the host (FP64) entry point: copies inside the timed region
    e2e_steps = args.e2e_steps or max(1, min(args.steps, 5))
    # host buffers as a MATLAB caller holds them: column-major complex128, output reused
    g_host = np.asfortranarray(gamma.cpu().numpy().astype(np.complex128))
    u_host = np.asfortranarray(u_meas.cpu().numpy().astype(np.complex128))
    grad_out = np.empty_like(g_host, order="F")
    op.vjp(g_host, u_host, out=grad_out)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        grad_h, loss_h = op.vjp(g_host, u_host, out=grad_out)
    t_e2e = time.perf_counter() - t0
    host_path = op.host_path()
    e2e = {"value": e2e_steps * B / t_e2e, "unit": "applies/s",
           "h2d_bytes_per_step": 16 * (P + N) * B, "d2h_bytes_per_step": 16 * P * B + 8 * B,
           "path": ("cui_born_vjp_host: the caller's FP64 host arrays read and written by device kernels through "
                    "the host page tables (Grace ATS over NVLink-C2C), VJP on the device in between"
                    + ("; the folded adjoint GEMM writes the FP64 gradient into the caller's array itself (one K "
                       "chunk per block)" if args.precision == "bf16x3-folded" and -(-P // 256) >= 4 * 152
                       else "")
                    if host_path == "direct" else
                    "cui_born_vjp_host: FP64 host buffers -> FP32 pinned staging -> H2D -> VJP -> D2H -> FP64"),
           "bytes": "FP64 complex host data crossing host<->device per step (gamma and u in, gradient and loss out)"}

    # roofline of the dominant contraction kernel
    clk = clocks.summary()
    roofline = roofline_of(args, op.info, kt, B, clk, p_used)
    info = op.info
    macs = info["contraction_macs"] * B

    line = {"metric": METRIC, "value": value, "unit": "applies/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "bf16x3 (split-BF16 operands, f32 accumulate)",
            "data": "synthetic (seeded)", "config": dict(workload_config(w, B), table_storage=TABLE_STORAGE[args.table_used]),
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "clocks": clk,
            "plan": {"build_s": t_build, "table_storage": op.table_storage,
                     "table_bytes": info["table_bytes"], "incident_bytes": info["incident_bytes"],
                     "workspace_bytes": info["workspace_bytes"], "complex_macs_per_apply": macs,
                     "channel_macs_per_apply": info["channel_macs"] * B,
                     "folded_bytes": info["folded_bytes"], "folded_sums": info["folded_sums"],
                     "folded_build_s": t_fold},
            "inputs": {"gamma": gamma_kind, "p_used_fraction": p_used,
                       "u": f"Phi gamma_true + complex Gaussian noise at {snr_db:.0f} dB SNR"},
            "loss": float(loss.sum().item()), "precision": args.precision, "autotune": autotune,
            "accuracy": accuracy,
            "device_status": op.device_status()}
    if args.fp32_steps > 0 and args.precision != "fp32":
        # the plain FP32 path of the same plan on the same inputs: the split-BF16 speed-up
        op.set_precision("fp32")
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(torch.cuda.current_stream())
        for _ in range(args.fp32_steps):
            step()
        e1.record(torch.cuda.current_stream())
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1) / args.fp32_steps
        v32 = world * B / (ms32 / 1e3)
        line["fp32_comparison"] = {"value": v32, "unit": "applies/s", "ms_per_step": ms32, "steps": args.fp32_steps,
                                   "speedup_bf16x3_over_fp32": value / v32,
                                   "rel_l2_grad_bf16x3_vs_fp32": (accuracy or {}).get("rel_l2_grad_vs_fp32")}
        if args.precision == "bf16x3-folded":
            # the element-contraction split-BF16 path of the same plan (tensor cores over slots and elements)
            op.set_precision("bf16x3")
            step()
            torch.cuda.synchronize()
            e0.record(torch.cuda.current_stream())
            for _ in range(args.fp32_steps):
                step()
            e1.record(torch.cuda.current_stream())
            torch.cuda.synchronize()
            mse = e0.elapsed_time(e1) / args.fp32_steps
            line["bf16x3_element_comparison"] = {"value": world * B / (mse / 1e3), "unit": "applies/s",
                                                 "ms_per_step": mse, "steps": args.fp32_steps,
                                                 "speedup_folded_over_element": value / (world * B / (mse / 1e3))}
        op.set_precision(args.precision)  # the timings below use the bench's own path again
    # received energies ||Phi e_p||^2 of the same plan (energy_rx, once per operator in the reference's solvers)
    op.energy_rx()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.current_stream())
    op.energy_rx()
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    line["energy_rx_ms"] = e0.elapsed_time(e1)
    if args.workload in ("2d-gradient", "2d-plain") and not args.no_greedy:
        line["greedy"] = time_greedy(op)
        line["greedy"]["precision"] = args.precision
    if B == 1 and args.n_freq is None:
        line["occupancy_sweep"] = occupancy_sweep(op)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            # the check needs the full workload: the oracle's sample takes its frequencies from the full list
            line["cpu_baseline"], check = cpu_baseline(args.workload, B, op if args.n_freq is None else None, w)
            line["accuracy"] = dict(line["accuracy"] or {}, fp64_oracle_sample=check)
        except Exception as exc:  # report, never hide
            line["cpu_baseline"] = {"value": None, "error": repr(exc)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    op.close()
    replicas_end(dist)


LASSO_CHECK_PROBLEM = 230  # the problem of the 256 with the least work: the CPU sample and the FP64 check


def lasso_macs(w) -> int:
    """Complex multiply-adds of one forward apply of a problem of the uneven batch (no receive
    mixing: every slot contracts all elements over all points)."""
    return len(w.f) * len(w.waves) * w.n_elements * w.n_points


def run_lasso(args):
    """Uneven-batch solver loop: all seeded problems (default 256), ``--lasso-iters``
    proximal-gradient LASSO iterations each (forward, residual, adjoint, soft threshold).

    The problems' plans need more device memory together than one GPU holds (about 956 GB
    with the split-BF16 copies, 322 GB in FP32).  So they run in batches that fit a
    device-memory budget.  For each batch, in seeded order:

    - the batch's plans are built;
    - the iterations of all its problems are captured into one CUDA graph, the problems spread
      over ``--lasso-streams`` streams;
    - the graph is replayed once;
    - the solutions are read back and the plans freed before the next batch.

    A preparation pass comes first.  It is untimed, and it also runs every kernel of every
    problem.  For each problem it:

    - builds the plan once and synthesises the data on the device: u = Phi gamma_true + 25 dB
      noise, lambda = 0.05 ||Phi^H u||_inf, step = 0.9 / ||Phi||^2 from 8 power iterations;
    - picks the path, with the per-plan autotuner by default;
    - measures the plan's device bytes on each path;
    - keeps u in pinned host memory (FP64).

    One step = one pass over all problems.  ``value`` = problems x iterations / the summed
    graph-replay time (CUDA events, every plan of the batch resident).  ``e2e`` = the same count
    / the pass's wall time, with every plan rebuilt, u copied from the host, the graphs captured
    and replayed, and the solutions copied back.  With several replicas the problems are split
    over them (they are independent); the job is fixed, so the scaling is strong.
    """
    import numpy as np
    import torch

    world, rank, local = dist_env()
    dist = replicas_begin(world)
    torch.cuda.set_device(local)
    from comp_ui_toolbox_gb300 import OperatorBorn, launch_count
    from comp_ui_toolbox_gb300.workloads import lasso_batch

    probs = lasso_batch(args.lasso_problems)
    mine = list(range(rank, len(probs), world))
    n_it = args.lasso_iters
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    budget = int(args.lasso_budget_gb * 1e9) if args.lasso_budget_gb else int(0.85 * free0)

    def used_bytes(reserved0, free_before):
        torch.cuda.synchronize()
        return (free_before - torch.cuda.mem_get_info()[0]) - (torch.cuda.memory_reserved() - reserved0)

    # ---- preparation pass (untimed) ----
    t0 = time.perf_counter()
    prep = {}
    for i in mine:
        w = probs[i]
        torch.cuda.synchronize()
        f_before, r_before = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
        op = OperatorBorn.from_setup(**w.setup_kwargs(), device=local, max_objects=1)
        g_true = torch.from_numpy(w.gamma(n_objects=1).astype(np.complex64)).cuda()
        u = op.forward(g_true)
        gen = torch.Generator(device="cuda").manual_seed(11 + i)
        noise = torch.randn(u.shape, dtype=torch.complex64, device="cuda", generator=gen)
        u = u + noise * (u.abs().pow(2).mean().sqrt() / noise.abs().pow(2).mean().sqrt()) * 10 ** (-25 / 20)
        L = op.norm_estimate(8)
        lam = 0.05 * float(op.adjoint(u).abs().max())
        rec = {"lam": lam, "step": 0.9 / L}
        uc = u.t().contiguous()
        lam_t = torch.tensor([lam], dtype=torch.float32, device="cuda")
        gtmp = torch.zeros((1, op.n_points), dtype=torch.complex64, device="cuda")
        op.lasso_(gtmp, uc, lam_t, rec["step"], 1)  # the FP32 path's workspaces exist before the bytes are read
        rec["bytes_fp32"] = used_bytes(r_before, f_before)
        if args.precision == "auto":
            tu = op.autotune(1)
            rec.update(precision=tu["precision"], shapes=tu["launch_shapes"])
        else:
            op.set_precision(args.precision)
            rec.update(precision=args.precision, shapes=None)
        op.lasso_(gtmp, uc, lam_t, rec["step"], 1)
        rec["bytes"] = used_bytes(r_before, f_before)
        rec["u_host"] = u.reshape(-1).to(torch.complex128).cpu().pin_memory()
        op.close()
        del u, uc, gtmp, noise, g_true
        prep[i] = rec
    torch.cuda.empty_cache()
    t_prep = time.perf_counter() - t0

    def batches(key):
        out, cur, acc = [], [], 0
        for i in mine:
            b = prep[i][key] + (64 << 20)  # + graph and stream bookkeeping
            if cur and acc + b > budget:
                out.append(cur)
                cur, acc = [], 0
            cur.append(i)
            acc += b
        if cur:
            out.append(cur)
        return out

    streams = [torch.cuda.Stream() for _ in range(max(1, args.lasso_streams))]

    def solve_pass(fp32: bool, objective=False):
        key = "bytes_fp32" if fp32 else "bytes"
        st = {"build_s": 0.0, "h2d_s": 0.0, "capture_s": 0.0, "solve_ms": 0.0, "d2h_s": 0.0, "kernel_nodes": 0,
              "batches": [], "h2d_bytes": 0, "d2h_bytes": 0}
        sols, obj = {}, {}
        t_obj = 0.0
        torch.cuda.synchronize()
        t_pass = time.perf_counter()
        for batch in batches(key):
            t = time.perf_counter()
            ops = []
            for i in batch:
                op = OperatorBorn.from_setup(**probs[i].setup_kwargs(), device=local, max_objects=1)
                p = "fp32" if fp32 else prep[i]["precision"]
                op.set_precision(p)
                sh = prep[i]["shapes"]
                if p == "bf16x3" and sh:
                    op.set_launch_shapes(*[v if isinstance(v, int) else 0
                                           for v in (sh["narrow_tiles"], sh["fwd_blocks"], sh["adj_blocks"])])
                ops.append(op)
            torch.cuda.synchronize()
            st["build_s"] += time.perf_counter() - t
            t = time.perf_counter()
            us = [prep[i]["u_host"].to("cuda", non_blocking=True) for i in batch]
            us = [u.to(torch.complex64).reshape(1, -1).contiguous() for u in us]
            torch.cuda.synchronize()
            st["h2d_s"] += time.perf_counter() - t
            st["h2d_bytes"] += sum(16 * u.numel() for u in us)
            t = time.perf_counter()
            lams = [torch.tensor([prep[i]["lam"]], dtype=torch.float32, device="cuda") for i in batch]
            gs = [torch.zeros((1, op.n_points), dtype=torch.complex64, device="cuda") for op in ops]
            for op, g, u, lam, i in zip(ops, gs, us, lams, batch):  # first use outside the capture
                op.lasso_(g, u, lam, prep[i]["step"], 1)
            torch.cuda.synchronize()
            for g in gs:
                g.zero_()
            n0 = launch_count()
            graph = torch.cuda.CUDAGraph()
            cap = torch.cuda.Stream()
            with torch.cuda.graph(graph, stream=cap):
                for k, (op, g, u, lam, i) in enumerate(zip(ops, gs, us, lams, batch)):
                    s = streams[k % len(streams)]
                    s.wait_stream(cap)
                    with torch.cuda.stream(s):
                        op.lasso_(g, u, lam, prep[i]["step"], n_it)
                for s in streams:
                    cap.wait_stream(s)
            nodes = launch_count() - n0
            st["kernel_nodes"] += nodes
            torch.cuda.synchronize()
            st["capture_s"] += time.perf_counter() - t
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            graph.replay()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            st["solve_ms"] += ms
            t = time.perf_counter()
            for i, g in zip(batch, gs):
                sols[i] = g.reshape(-1).cpu().numpy().astype(np.complex128)
                st["d2h_bytes"] += 16 * g.numel()
            st["d2h_s"] += time.perf_counter() - t
            if objective:
                t = time.perf_counter()
                for op, g, u, lam, i in zip(ops, gs, us, lams, batch):
                    r = op.forward(g.t().contiguous()) - u.t()
                    obj[i] = float(0.5 * r.abs().pow(2).sum() + lam.item() * g.abs().sum())
                t_obj += time.perf_counter() - t
            st["batches"].append({"problems": len(batch), "gb": sum(prep[i][key] for i in batch) / 1e9,
                                  "graph_nodes": nodes, "replay_ms": ms})
            del graph, gs, us, lams
            for op in ops:
                op.close()
            torch.cuda.empty_cache()
        st["wall_s"] = time.perf_counter() - t_pass - t_obj
        return st, sols, obj

    with ClockSampler(local) as clocks:
        replicas_barrier(dist)
        clocks.mark_start()
        st, sols, obj = solve_pass(False, objective=True)
        clocks.mark_end()
    replicas_barrier(dist)
    ms = replicas_max_ms(dist, st["solve_ms"], device="cuda")
    wall_ms = replicas_max_ms(dist, 1e3 * st["wall_s"], device="cuda")
    n_total = len(probs) * n_it
    value = n_total / (ms / 1e3)
    st32 = sols32 = None
    if args.fp32_steps > 0 and args.precision != "fp32":
        st32, sols32, _ = solve_pass(True)
    precs = [prep[i]["precision"] for i in mine]
    line = {"metric": METRIC, "value": value, "unit": "applies/s", "n_gpus": world, "steps": 1,
            "warmup": 1, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None,
            "dtype": {"fp32": "f32", "auto": "per problem: f32 or bf16x3 (autotuned)"}.get(
                args.precision, "bf16x3 (split-BF16 operands, f32 accumulate)"),
            "data": "synthetic (seeded)",
            "config": {"workload": f"2d-lasso: all {len(probs)} seeded uneven problems (FOV side 128-512, 1-16 "
                                   f"waves, 32-256 frequencies, 64/128 elements), {n_it} proximal-gradient LASSO "
                                   f"iterations each; batches within a {budget / 1e9:.0f} GB device-memory budget, "
                                   f"one CUDA graph per batch over {len(streams)} streams; one step = one pass over "
                                   f"all problems",
                       "problems": len(probs), "iterations": n_it,
                       "total_complex_macs_per_iteration": int(2 * sum(lasso_macs(probs[i]) for i in mine)),
                       "l2": "inputs larger than L2 (tables and incident fields, GBs per batch, re-read every "
                             "iteration)"},
            "step_definition": "one pass over all problems: ms_per_step = summed graph-replay time of the batches "
                               "(CUDA events); value = problems x iterations / that time",
            "warmup_definition": "the preparation pass: every problem's plan built once, its data synthesised, "
                                 "its path autotuned, its kernels run",
            "gpu_launches": st["kernel_nodes"],
            "graph": {"batches": st["batches"], "kernel_nodes": st["kernel_nodes"]},
            "job": {"wall_s": st["wall_s"], "plan_build_s": st["build_s"], "h2d_s": st["h2d_s"],
                    "capture_s": st["capture_s"], "replay_s": st["solve_ms"] / 1e3, "d2h_s": st["d2h_s"],
                    "preparation_pass_s": t_prep},
            "clocks": clocks.summary(), "precision": args.precision,
            "paths": {"bf16x3": precs.count("bf16x3"), "fp32": precs.count("fp32")},
            "objective_after": {"mean": float(np.mean(list(obj.values()))), "problems": len(obj)},
            "e2e": {"value": n_total / (wall_ms / 1e3), "unit": "applies/s",
                    "h2d_bytes_per_step": st["h2d_bytes"], "d2h_bytes_per_step": st["d2h_bytes"],
                    "path": "one pass: every plan rebuilt from its setup, FP64 measured data from pinned host "
                            "memory, one graph per batch captured and replayed, solutions back to the host"}}
    if st32 is not None:
        rels = [float(np.linalg.norm(sols[i] - sols32[i]) / max(np.linalg.norm(sols32[i]), 1e-30)) for i in mine]
        line["fp32_comparison"] = {"value": n_total / (st32["solve_ms"] / 1e3), "unit": "applies/s",
                                   "ms_per_step": st32["solve_ms"], "wall_s": st32["wall_s"],
                                   "batches": len(st32["batches"]),
                                   "speedup_over_fp32": st32["solve_ms"] / st["solve_ms"],
                                   "max_rel_l2_solution_vs_fp32": max(rels),
                                   "median_rel_l2_solution_vs_fp32": float(np.median(rels))}
    if rank == 0 and world == 1 and not args.no_cpu_baseline and LASSO_CHECK_PROBLEM in prep:
        line["cpu_baseline"], line["fp64_oracle_check"] = lasso_cpu_baseline(
            probs, LASSO_CHECK_PROBLEM, prep[LASSO_CHECK_PROBLEM], n_it,
            sols[LASSO_CHECK_PROBLEM], sols32[LASSO_CHECK_PROBLEM] if sols32 else None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    replicas_end(dist)


def lasso_problem_oracle(w):
    from oracle.lasso_split import lasso_problem_config
    return lasso_problem_config(w.n_points_axis[0], w.n_elements, w.f, [a[0] for _, a in w.waves], w.density,
                                w.seed, w.name)


def lasso_cpu_baseline(probs, i, rec, n_it, sol, sol32):
    """The FP64 oracle's ISTA (split over frequencies, one spawn worker per host core) on problem
    ``i`` with the device's data: timed, scaled to the whole batch by multiply-adds, and its
    solution compared with the device's."""
    import numpy as np
    from oracle.lasso_split import FrequencySplitOracle
    w = probs[i]
    with FrequencySplitOracle(lasso_problem_oracle(w)) as orc:
        t0 = time.perf_counter()
        g, _ = orc.lasso(rec["u_host"].numpy(), rec["lam"], rec["step"], n_it)
        t = time.perf_counter() - t0
        cores = len(orc.f_sets)
    scale = sum(lasso_macs(p) for p in probs) / lasso_macs(w)
    value = len(probs) * n_it / (t * scale)
    g = g[:, 0]
    rel = lambda x: float(np.linalg.norm(x - g) / np.linalg.norm(g))
    base = {"value": value, "unit": "applies/s", "cores": cores, "kind": "port",
            "sample": f"problem {i} of the batch ({w.n_points_axis[0]}x{w.n_points_axis[1]} grid, {len(w.waves)} "
                      f"waves, {len(w.f)} frequencies, {w.n_elements} elements): {n_it} ISTA iterations of the FP64 "
                      f"oracle (oracle.solvers.lasso_ista), frequencies split over {cores} spawn processes; whole-batch "
                      f"rate = sample rate x that problem's multiply-adds / all problems' ({scale:.0f}x)",
            "seconds_sample": t}
    check = {"problem": i, "iterations": n_it, "rel_l2_solution_vs_fp64_ista": rel(sol),
             "rel_l2_fp32_solution_vs_fp64_ista": rel(sol32) if sol32 is not None else None,
             "what": "device LASSO solution after all iterations vs the FP64 oracle's ISTA on the same u, lambda, step"}
    return base, check


def run_reference_lasso(args):
    """Reference arm of the uneven batch: the FP64 oracle's ISTA on the problem with the least work
    (its own data: FP64 forward of gamma_true + 25 dB noise, lambda and step from the oracle), split
    over frequencies across the host cores; each step times ``REF_LASSO_ITERS`` iterations and
    ``value`` scales them to the whole batch by multiply-adds."""
    import numpy as np
    from comp_ui_toolbox_gb300.workloads import lasso_batch
    from oracle.lasso_split import FrequencySplitOracle
    probs = lasso_batch(args.lasso_problems)
    i = LASSO_CHECK_PROBLEM if LASSO_CHECK_PROBLEM < len(probs) else 0
    w = probs[i]
    t0 = time.perf_counter()
    with FrequencySplitOracle(lasso_problem_oracle(w)) as orc:
        u0 = orc.forward(w.gamma(n_objects=1).real + 0j)
        rng = np.random.default_rng(1000 + i)
        noise = rng.standard_normal(u0.shape) + 1j * rng.standard_normal(u0.shape)
        u = u0 + noise * (np.linalg.norm(u0) / np.linalg.norm(noise)) * 10 ** (-25 / 20)
        lam = 0.05 * float(np.abs(orc.adjoint(u)).max())
        x = rng.standard_normal((orc.P, 1)) + 0j
        for _ in range(8):  # power iterations on Phi^H Phi
            y = orc.adjoint(orc.forward(x))
            L = float(np.linalg.norm(y) / np.linalg.norm(x))
            x = y / np.linalg.norm(y)
        step = 0.9 / L
        times = []
        g = None
        for _ in range(args.warmup + args.steps):
            t = time.perf_counter()
            g, _ = lasso_ista_from(orc, u, lam, step, REF_LASSO_ITERS, g)
            times.append(time.perf_counter() - t)
        cores = len(orc.f_sets)
    wall = time.perf_counter() - t0
    timed = sorted(times[args.warmup:])
    t_step = timed[len(timed) // 2]
    scale = sum(lasso_macs(p) for p in probs) / lasso_macs(w)
    value = len(probs) * REF_LASSO_ITERS / (t_step * scale)
    sample = (f"problem {i} of the batch: {REF_LASSO_ITERS} ISTA iterations of the FP64 oracle per step, frequencies "
              f"split over {cores} spawn processes; whole-batch rate = sample rate x that problem's multiply-adds / "
              f"all problems' ({scale:.0f}x)")
    line = {"metric": METRIC, "value": value, "unit": "applies/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"2d-lasso: all {len(probs)} seeded uneven problems, {args.lasso_iters} "
                                   f"proximal-gradient LASSO iterations each", "problems": len(probs)},
            "impl": "reference", "extrapolated": True, "scale_factor": scale, "wall_s": wall,
            "cpu_baseline": {"value": value, "unit": "applies/s", "cores": cores, "kind": "port",
                             "host_cores": os.cpu_count(), "sample": sample},
            "e2e": {"value": value, "unit": "applies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


REF_LASSO_ITERS = 10


def lasso_ista_from(orc, u, lam, step, n_iter, gamma0):
    from oracle.solvers import lasso_ista
    return lasso_ista(None, u, lam, step, n_iter, gamma0=gamma0, forward=orc.forward, adjoint=orc.adjoint,
                      n_points=orc.P)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_as_replicas(args.gpus))
    if args.precision is None:
        args.precision = {"2d-batched": "bf16x3-folded", "3d": "fp32"}.get(args.workload, "auto")
    if args.table_storage is None:
        args.table_storage = {"3d": "streamed"}.get(args.workload, "auto")
    if args.impl == "reference":
        if args.workload == "2d-lasso":
            if int(os.environ.get("RANK", "0")) == 0:
                run_reference_lasso(args)
        else:
            run_reference(args)
    elif args.workload == "2d-lasso":
        run_lasso(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
