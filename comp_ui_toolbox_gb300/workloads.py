"""Synthetic benchmark workloads of the Born operator (caller-side inputs).

The reference benchmarks its operator on no public dataset; these seeded
synthetic setups stand in with the stated shapes, sizes and distributions:

* ``2d-plain``: 2D, 128-element linear array (0.3048 mm pitch, L14-5/38), one
  quasi-plane wave at 0 deg, 64 frequencies over 2.5-5.5 MHz, lossless water,
  256x256 FOV at 76.2 um from 5 mm, identity receive mixing, gamma real with
  2% N(0,1) nonzeros;
* ``2d-gradient``: same array, 11 quasi-plane waves -20..20 deg, 192
  frequencies over 2-6 MHz, time-causal absorption 0.5 dB/(MHz cm) at 4 MHz,
  512x512 FOV, gamma 5%; the gradient of 0.5||Phi gamma - u||^2;
* ``2d-batched``: 512x512, 128 frequencies over 2.5-5.5 MHz, 16 waves with
  random apodization in [-1, 1] and random delays in [0, 1] us, 32 receive
  mixes with random +-1 weights, 64 gamma columns at 3% density;
* ``3d``: 32x32 matrix array at 0.3 mm, 5 quasi-plane waves -10..10 deg
  azimuth, 64 frequencies, 128^3 FOV at 0.1 mm from 5 mm, absorbing, gamma 1%;
* ``2d-lasso`` (:func:`lasso_batch`): independent 2D problems of seeded sizes
  (FOV side in {128, 192, 256, 384, 512} at 76.2 um, 1-16 quasi-plane waves
  over -20..20 deg, 32-256 frequencies over 2.5-5.5 MHz, 64 or 128 elements at
  0.3048 mm pitch, lossless), gamma_true 2%, data with 25 dB noise, each
  solved by 50 proximal-gradient LASSO iterations.

The wave synthesis restates the reference's delay laws: quasi-plane-wave
delays ``<x_e, e_theta>/c`` shifted to zero minimum
(``+scattering/+sequences/+syntheses/+deterministic/qpw.m:96-97``), delays
quantised to the 80 MHz transmit clock (``+scattering/+sequences/+setups/setup.m:22``,
``:625``) and normal velocities ``excitation * impulse response * exp(-2 pi j f tau)``
(``+scattering/+sequences/+settings/+controls/tx.m:284``, ``setup.m:630-635``).
"""

from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np

T_CLK = 1.0 / 80e6
PITCH_L14 = 304.8e-6
WIDTH_L14 = 279.8e-6
DX_2D = 76.2e-6
LOSSLESS = {"kind": "none", "c": 1500.0}
TISSUE = {"kind": "time_causal", "c": 1500.0, "constant_db": 0.0, "slope_db": 0.5, "exponent": 1.0,
          "f_ref": 4e6, "dispersion": True}


@dataclasses.dataclass
class Workload:
    name: str
    n_points_axis: tuple
    delta_axis: tuple
    z_start: float
    n_elements_axis: tuple
    pitch_axis: tuple
    width_axis: tuple
    n_face_axis: tuple
    absorption: dict
    f: np.ndarray
    waves: list               # ("qpw", angles_deg) or ("rad", seed)
    mixing: str = "identity"  # or "pm1"
    n_mixes: int = 0
    mix_seed: int = 0
    n_objects: int = 1
    density: float = 0.02
    seed: int = 0
    aa_beta: Optional[float] = 0.5

    @property
    def n_elements(self) -> int:
        return int(np.prod(self.n_elements_axis))

    @property
    def n_points(self) -> int:
        return int(np.prod(self.n_points_axis))

    def element_centers(self) -> np.ndarray:
        axes = [(np.arange(n) - (n - 1) / 2.0) * p for n, p in zip(self.n_elements_axis, self.pitch_axis)]
        mesh = np.meshgrid(*axes, indexing="ij")
        return np.stack([m.reshape(-1, order="F") for m in mesh], axis=1)

    def wave_vd(self, wave) -> np.ndarray:
        """Normal velocities v_d(f, e) of one wave."""
        kind = wave[0]
        E = self.n_elements
        if kind == "qpw":
            ang = np.deg2rad(np.asarray(wave[1], dtype=np.float64))
            tau = self.element_centers() @ np.sin(ang)[: len(self.n_elements_axis)] / self.absorption["c"]
            tau = tau - tau.min()
            apod = np.ones(E)
        elif kind == "rad":
            rng = np.random.default_rng(wave[1])
            apod = rng.uniform(-1.0, 1.0, E)
            tau = rng.uniform(0.0, 1e-6, E)
        else:
            raise ValueError(kind)
        tau = np.round(tau / T_CLK) * T_CLK
        f = self.f
        fc = 0.5 * (f.min() + f.max())
        spectrum = np.exp(-0.5 * ((f - fc) / (0.4 * fc)) ** 2)
        return spectrum[:, None] * apod[None, :] * np.exp(-2j * np.pi * f[:, None] * tau[None, :])

    def mix_weights(self) -> np.ndarray:
        E = self.n_elements
        if self.mixing == "identity":
            return np.eye(E)
        rng = np.random.default_rng(self.mix_seed)
        return np.where(rng.random((self.n_mixes, E)) < 0.5, -1.0, 1.0)

    def setup_kwargs(self) -> dict:
        """Keyword arguments of :meth:`OperatorBorn.from_setup`."""
        weights = self.mix_weights()
        F = len(self.f)
        mixes = []
        for m in range(weights.shape[0]):
            active = np.nonzero(weights[m])[0]
            mixes.append({"f_idx": np.arange(F), "active": active,
                          "response": np.repeat(weights[m, active][None, :], F, axis=0).astype(np.complex128)})
        waves = [{"f_idx": np.arange(F), "v_d": self.wave_vd(w), "mixes": mixes} for w in self.waves]
        return dict(n_points_axis=self.n_points_axis, delta_axis=self.delta_axis, z_start=self.z_start,
                    n_elements_axis=self.n_elements_axis, pitch_axis=self.pitch_axis, width_axis=self.width_axis,
                    n_face_axis=self.n_face_axis, absorption=self.absorption, f_unique=self.f, waves=waves,
                    aa_tx_beta=self.aa_beta, aa_rx_beta=self.aa_beta)

    def gamma(self, seed: Optional[int] = None, n_objects: Optional[int] = None) -> np.ndarray:
        """Seeded sparse fluctuations: ``density`` nonzeros per column, N(0,1) values."""
        rng = np.random.default_rng(self.seed if seed is None else seed)
        P = self.n_points
        B = self.n_objects if n_objects is None else n_objects
        g = np.zeros((P, B), dtype=np.complex128)
        nnz = max(1, int(round(self.density * P)))
        for b in range(B):
            idx = rng.choice(P, nnz, replace=False)
            g[idx, b] = rng.standard_normal(nnz)
        return g


def _qpw_range(lo, hi, step):
    return [("qpw", (float(a),)) for a in np.arange(lo, hi + step / 2, step)]


def workload(name: str) -> Workload:
    if name == "2d-plain":
        return Workload(name, (256, 256), (DX_2D, DX_2D), 5e-3, (128,), (PITCH_L14,), (WIDTH_L14,), (1,), LOSSLESS,
                        np.linspace(2.5e6, 5.5e6, 64), [("qpw", (0.0,))], density=0.02, seed=1000)
    if name == "2d-gradient":
        return Workload(name, (512, 512), (DX_2D, DX_2D), 5e-3, (128,), (PITCH_L14,), (WIDTH_L14,), (1,), TISSUE,
                        np.linspace(2.0e6, 6.0e6, 192), _qpw_range(-20, 20, 4), density=0.05, seed=1001)
    if name == "2d-batched":
        return Workload(name, (512, 512), (DX_2D, DX_2D), 5e-3, (128,), (PITCH_L14,), (WIDTH_L14,), (1,), LOSSLESS,
                        np.linspace(2.5e6, 5.5e6, 128), [("rad", 2000 + i) for i in range(16)], mixing="pm1",
                        n_mixes=32, mix_seed=2100, n_objects=64, density=0.03, seed=1002)
    if name == "3d":
        return Workload(name, (128, 128, 128), (1e-4, 1e-4, 1e-4), 5e-3, (32, 32), (3e-4, 3e-4), (2.7e-4, 2.7e-4),
                        (1, 1), TISSUE, np.linspace(2.5e6, 5.5e6, 64),
                        [("qpw", (float(a), 0.0)) for a in (-10, -5, 0, 5, 10)], density=0.01, seed=1003)
    raise KeyError(name)


def lasso_problem(i: int, seed: int = 4000) -> Workload:
    """Problem ``i`` of the seeded uneven batch (sizes drawn independently per problem)."""
    rng = np.random.default_rng(seed + i)
    side = int(rng.choice([128, 192, 256, 384, 512]))
    n_waves = int(rng.integers(1, 17))
    n_f = int(rng.integers(32, 257))
    n_el = int(rng.choice([64, 128]))
    angles = np.linspace(-20.0, 20.0, n_waves) if n_waves > 1 else np.array([0.0])
    return Workload(f"2d-lasso[{i}]", (side, side), (DX_2D, DX_2D), 5e-3, (n_el,), (PITCH_L14,), (WIDTH_L14,), (1,),
                    LOSSLESS, np.linspace(2.5e6, 5.5e6, n_f), [("qpw", (float(a),)) for a in angles],
                    density=0.02, seed=seed + 1000 + i)


def lasso_batch(n_problems: int, seed: int = 4000) -> list:
    """The first ``n_problems`` problems of the seeded uneven batch."""
    return [lasso_problem(i, seed) for i in range(n_problems)]


def plan_bytes_estimate(w: Workload, tensor_cores: bool = True) -> int:
    """Device bytes a plan of ``w`` holds (tables, incident fields, their split-BF16 copies)."""
    Nx, Nz = w.n_points_axis[0], w.n_points_axis[-1]
    F, W, E = len(w.f), len(w.waves), w.n_elements
    table = F * Nz * (Nx + (E - 1) * 4) * 8
    incident = W * F * w.n_points * 8
    return int(table * (2 if tensor_cores else 1) + incident * (3.2 if tensor_cores else 1))


NAMES = ("2d-plain", "2d-gradient", "2d-batched", "3d")
