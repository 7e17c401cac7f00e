"""Seeded synthetic workloads for the Born operator (test infrastructure).

Defines the five benchmark workloads (2D plain, 2D with gradient, 2D batched
random-apodization, 3D matrix array, uneven solver batch) at full size and at
reduced test sizes, and builds the oracle's operator tables for them.

The reference takes no public dataset on this path; every input here is a
seeded synthetic stand-in with the stated shapes, sizes and distributions.
"""

from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

from .born_oracle import (
    Absorption, Measurement, Mix, OperatorTables, Setup, face_symmetric, incident_field, lateral_table,
    qpw_delays, quantize_delays, shift_lateral, transfer_function, wavenumbers,
)

# L14-5/38 geometry (+scattering/+sequences/+setups/+transducers/parameters_L14_5_38.m)
PITCH_L14 = 304.8e-6
WIDTH_L14 = 279.8e-6
DX_2D = 76.2e-6


@dataclasses.dataclass
class Wave:
    """Incident wave: ``kind`` 'qpw' (steering angles in degrees, lateral
    axes) or 'rad' (random apodization in [-1, 1] and random delays in
    [0, max_delay], seeded), with the subset of global frequencies it uses."""

    kind: str
    angles_deg: tuple = (0.0,)
    seed: int = 0
    max_delay: float = 1e-6
    f_subset: Optional[np.ndarray] = None


@dataclasses.dataclass
class BornConfig:
    name: str
    setup: Setup
    f: np.ndarray
    waves: list
    mixing: str = "identity"  # 'identity' or 'pm1'
    n_mixes: int = 0
    mix_seed: int = 0
    mix_f_stride: int = 1      # >1: mixes use every n-th measurement frequency
    n_objects: int = 1
    density: float = 0.02
    seed: int = 0
    band: Optional[tuple] = None  # (f_min, f_max) of the excitation spectrum; None: the range of f

    @property
    def n_waves(self):
        return len(self.waves)


def _setup_2d(n_x, n_z, n_el, absorption, n_face=1, dx=DX_2D, z_start=5e-3):
    return Setup(n_points_axis=(n_x, n_z), delta_axis=(dx, dx), z_start=z_start,
                 n_elements_axis=(n_el,), pitch_axis=(PITCH_L14 if dx == DX_2D else 4 * dx,),
                 width_axis=(WIDTH_L14 if dx == DX_2D else 3.7 * dx,), n_face_axis=(n_face,),
                 absorption=absorption)


LOSSLESS = Absorption("none", 1500.0)
TISSUE = Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True)


def qpw_angles(lo, hi, step):
    return tuple(float(a) for a in np.arange(lo, hi + step / 2, step))


def config(name: str) -> BornConfig:
    """Full-size workload by name: c0 ... c3 (c4 is built by :func:`uneven_batch`)."""
    if name == "c0":
        return BornConfig("c0: 2D plain, 256x256, 64 f, 128 ch, 1 QPW",
                          _setup_2d(256, 256, 128, LOSSLESS), np.linspace(2.5e6, 5.5e6, 64),
                          [Wave("qpw", (0.0,))], density=0.02, seed=1000)
    if name == "c1":
        return BornConfig("c1: 2D gradient, 512x512, 192 f, 128 ch, 11 QPW, absorbing",
                          _setup_2d(512, 512, 128, TISSUE), np.linspace(2.0e6, 6.0e6, 192),
                          [Wave("qpw", (a,)) for a in qpw_angles(-20, 20, 4)], density=0.05, seed=1001)
    if name == "c2":
        return BornConfig("c2: 2D batched, 512x512, 128 f, 16 RA waves -> 32 mixes, 64 columns",
                          _setup_2d(512, 512, 128, LOSSLESS), np.linspace(2.5e6, 5.5e6, 128),
                          [Wave("rad", seed=2000 + i) for i in range(16)], mixing="pm1", n_mixes=32,
                          mix_seed=2100, n_objects=64, density=0.03, seed=1002)
    if name == "c3":
        s = Setup(n_points_axis=(128, 128, 128), delta_axis=(1e-4, 1e-4, 1e-4), z_start=5e-3,
                  n_elements_axis=(32, 32), pitch_axis=(3e-4, 3e-4), width_axis=(2.7e-4, 2.7e-4),
                  n_face_axis=(1, 1), absorption=TISSUE)
        return BornConfig("c3: 3D, 128^3, 64 f, 32x32 array, 5 QPW", s, np.linspace(2.5e6, 5.5e6, 64),
                          [Wave("qpw", (a, 0.0)) for a in (-10, -5, 0, 5, 10)], density=0.01, seed=1003)
    raise KeyError(name)


def small_config(name: str) -> BornConfig:
    """Reduced test-size variants that keep each workload's structure."""
    if name == "c0":   # FOV narrower than the array: symmetric index map out of range
        return BornConfig("c0-small", _setup_2d(40, 20, 16, LOSSLESS), np.linspace(2.5e6, 5.5e6, 8),
                          [Wave("qpw", (0.0,))], density=0.05, seed=11)
    if name == "c1":   # FOV wider than the array, absorbing, several waves
        return BornConfig("c1-small", _setup_2d(64, 24, 16, TISSUE), np.linspace(2.0e6, 6.0e6, 12),
                          [Wave("qpw", (a,)) for a in (-8.0, 0.0, 8.0)], density=0.05, seed=12)
    if name == "c2":
        return BornConfig("c2-small", _setup_2d(64, 16, 16, LOSSLESS), np.linspace(2.5e6, 5.5e6, 8),
                          [Wave("rad", seed=200 + i) for i in range(4)], mixing="pm1", n_mixes=5,
                          mix_seed=210, n_objects=6, density=0.03, seed=13)
    if name == "five":  # five waves per frequency: the FP32 kernels' 5-column instantiation
        return BornConfig("five-small", _setup_2d(64, 24, 16, TISSUE), np.linspace(2.0e6, 6.0e6, 8),
                          [Wave("qpw", (a,)) for a in (-8.0, -4.0, 0.0, 4.0, 8.0)], density=0.05, seed=16)
    if name == "ragged":  # uneven frequency subsets per wave and per mix
        f = np.linspace(2.5e6, 5.5e6, 10)
        waves = [Wave("qpw", (-6.0,), f_subset=np.array([0, 1, 2, 3, 5, 7, 9])),
                 Wave("qpw", (4.0,), f_subset=np.array([2, 4, 6, 8])),
                 Wave("rad", seed=5, f_subset=np.arange(10))]
        return BornConfig("ragged-small", _setup_2d(52, 14, 12, TISSUE), f, waves, mixing="pm1",
                          n_mixes=3, mix_seed=7, mix_f_stride=2, n_objects=3, density=0.1, seed=14)
    if name == "c3":
        s = Setup(n_points_axis=(12, 10, 6), delta_axis=(1e-4, 1e-4, 1e-4), z_start=3e-3,
                  n_elements_axis=(4, 3), pitch_axis=(3e-4, 3e-4), width_axis=(2.7e-4, 2.7e-4),
                  n_face_axis=(1, 1), absorption=TISSUE)
        return BornConfig("c3-small", s, np.linspace(2.5e6, 5.5e6, 4),
                          [Wave("qpw", (a, 0.0)) for a in (-10, 0, 10)], density=0.05, seed=15)
    raise KeyError(name)


# --------------------------------------------------------------------------
def excitation_spectrum(f: np.ndarray, band=None) -> np.ndarray:
    """Smooth synthetic excitation x impulse-response spectrum (Gaussian in f, centred on the band:
    the range of ``f`` unless ``band`` = (f_min, f_max) is given)."""
    lo, hi = (f.min(), f.max()) if band is None else band
    fc = 0.5 * (lo + hi)
    return np.exp(-0.5 * ((f - fc) / (0.4 * fc)) ** 2)


def wave_vd(cfg: BornConfig, wave: Wave, f: np.ndarray) -> np.ndarray:
    """Normal velocities v_d(f, e) of one wave (``tx.m:284``, ``setup.m:600-635``)."""
    s = cfg.setup
    E = s.n_elements
    if wave.kind == "qpw":
        ang = np.deg2rad(np.asarray(wave.angles_deg, dtype=np.float64))
        e_lat = np.sin(ang)[: s.n_lat]
        tau = qpw_delays(s, e_lat)
        apod = np.ones(E)
    elif wave.kind == "rad":
        rng = np.random.default_rng(wave.seed)
        apod = rng.uniform(-1.0, 1.0, E)
        tau = rng.uniform(0.0, wave.max_delay, E)
    else:
        raise ValueError(wave.kind)
    tau = quantize_delays(tau)
    return excitation_spectrum(f, cfg.band)[:, None] * apod[None, :] * np.exp(-2j * np.pi * f[:, None] * tau[None, :])


def mix_weights(cfg: BornConfig):
    """(M, E) receive mixing weights: identity or seeded +-1."""
    E = cfg.setup.n_elements
    if cfg.mixing == "identity":
        return np.eye(E)
    rng = np.random.default_rng(cfg.mix_seed)
    return np.where(rng.random((cfg.n_mixes, E)) < 0.5, -1.0, 1.0)


def mix_layout(cfg: BornConfig, n_f_wave: int):
    """Per mix: (frequency indices into the wave's frequencies, active elements,
    receive responses R (F_mix, n_active))."""
    weights = mix_weights(cfg)
    out = []
    for m in range(weights.shape[0]):
        active = np.nonzero(weights[m])[0]
        if cfg.mix_f_stride > 1:
            mf = np.arange(m % 2, n_f_wave, cfg.mix_f_stride)
        else:
            mf = np.arange(n_f_wave)
        resp = np.repeat(weights[m, active][None, :], len(mf), axis=0).astype(np.complex128)
        out.append((mf, active, resp))
    return out


@dataclasses.dataclass
class BuiltOperator:
    """Oracle tables plus the lateral-offset form consumed by the CUDA path."""

    cfg: BornConfig
    op: OperatorTables
    table_rx: np.ndarray      # (F_u, Nz, [No_y,] No_x) receive table
    table_tx: np.ndarray      # transmit table (tx anti-aliasing filter)
    symmetric_valid: bool


def element_from_table(setup: Setup, table: np.ndarray, e: int) -> np.ndarray:
    """Element ``e``'s transfer function (F, P) read from a lateral table."""
    P = np.arange(setup.n_points)
    if setup.n_dims == 2:
        Nx = setup.n_points_axis[0]
        ix, iz = P % Nx, P // Nx
        o = ix - e * setup.ppp_axis[0] + (setup.n_elements_axis[0] - 1) * setup.ppp_axis[0]
        return table[:, iz, o]
    Nx, Ny, _ = setup.n_points_axis
    Ex, Ey = setup.n_elements_axis
    px, py = setup.ppp_axis
    ix, iy, iz = P % Nx, (P // Nx) % Ny, P // (Nx * Ny)
    ex, ey = e % Ex, e // Ex
    return table[:, iz, iy - ey * py + (Ey - 1) * py, ix - ex * px + (Ex - 1) * px]


def build(cfg: BornConfig, direct_elements: bool = False) -> BuiltOperator:
    """Build the oracle operator for a workload.

    The incident fields sum element transfer functions read from the
    transmit lateral table (identical to direct evaluation, which the oracle
    tests pin).  The receive side uses the reference's symmetric-grid
    representation (``h_ref`` + ``indices_grid_FOV_shift``) when its index
    map is in range, otherwise per-element transfer functions: evaluated
    directly when ``direct_elements`` is set, else read from the receive
    table.
    """
    s = cfg.setup
    f = np.asarray(cfg.f, dtype=np.float64)
    T_tx = lateral_table(s, f, s.aa_tx_beta)
    T_rx = T_tx if s.aa_tx_beta == s.aa_rx_beta else lateral_table(s, f, s.aa_rx_beta)
    k = wavenumbers(s, f)
    weights = mix_weights(cfg)
    measurements = []
    for wave in cfg.waves:
        f_idx = np.arange(len(f)) if wave.f_subset is None else np.asarray(wave.f_subset)
        fw = f[f_idx]
        v_d = wave_vd(cfg, wave, fw)
        p_in = incident_field(s, fw, v_d, lambda e: element_from_table(s, T_tx, e)[f_idx])
        mixes = []
        for mf, active, resp in mix_layout(cfg, len(f_idx)):
            kk = k[f_idx[mf]]
            # prefactors -dV k~^2 (setup.m:759) times the receive impulse-response DFT (sequence.m:623)
            mixes.append(Mix(f_idx=mf, active=active, pref=(-s.cell_volume * kk ** 2)[:, None] * resp))
        measurements.append(Measurement(f_idx=f_idx, p_incident=p_in, mixes=mixes))
    shift, valid = shift_lateral(s)
    valid = valid and face_symmetric(s)  # mirroring h_ref needs a face symmetric about its centroid
    op = OperatorTables(setup=s, f_unique=f, measurements=measurements)
    if valid:
        op.h_ref = transfer_function(s, f, 0, s.aa_rx_beta)
        op.shift = shift
    else:
        cache = {}

        def h_element(e):
            if e not in cache:
                cache[e] = (transfer_function(s, f, e, s.aa_rx_beta) if direct_elements
                            else element_from_table(s, T_rx, e))
            return cache[e]
        op.h_element = h_element
    return BuiltOperator(cfg=cfg, op=op, table_rx=T_rx, table_tx=T_tx, symmetric_valid=valid)


def make_gamma(cfg: BornConfig, seed: Optional[int] = None, n_objects: Optional[int] = None,
               complex_values: bool = False) -> np.ndarray:
    """Seeded sparse fluctuations: ``density`` nonzeros per column, N(0,1) values."""
    rng = np.random.default_rng(cfg.seed if seed is None else seed)
    P = cfg.setup.n_points
    B = cfg.n_objects if n_objects is None else n_objects
    g = np.zeros((P, B), dtype=np.complex128)
    nnz = max(1, int(round(cfg.density * P)))
    for b in range(B):
        idx = rng.choice(P, nnz, replace=False)
        vals = rng.standard_normal(nnz)
        if complex_values:
            vals = vals + 1j * rng.standard_normal(nnz)
        g[idx, b] = vals
    return g


def add_noise(u: np.ndarray, snr_db: float, seed: int) -> np.ndarray:
    """Complex Gaussian noise at the given SNR (per column)."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(u.shape) + 1j * rng.standard_normal(u.shape)
    p_sig = np.mean(np.abs(u) ** 2, axis=0, keepdims=True)
    p_noise = np.mean(np.abs(noise) ** 2, axis=0, keepdims=True)
    return u + noise * np.sqrt(p_sig / p_noise * 10 ** (-snr_db / 10))
