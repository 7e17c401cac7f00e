"""FP64 restatement of the reference Born operator and its tables.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the oracle the CUDA
library's results are checked against, never the thing measured or shipped.

All citations are paths inside the reference project
(mschiffn/comp_ui_toolbox).  Conventions kept from the reference:

* grids are column-major: the first lateral axis (x) runs fastest, the axial
  axis (z) is the last axis (``+math/grid_regular.m:140-260``);
* lateral axes of the field of view (FOV) are centred on the array axis, the
  axial axis starts at ``z_start``; a grid built from an interval of length
  ``N*delta`` has its points at the cell centres
  (``+scattering/+sequences/+setups/+geometry/orthotope.m:140-146``);
* element ``e`` of an ``Ex x Ey`` array has linear index ``ex + Ex*ey``;
* complex numbers are FP64 throughout.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Callable, Optional, Sequence

import numpy as np
from scipy.special import hankel2

__all__ = [
    "Setup", "Absorption", "Mix", "Measurement", "OperatorTables",
    "wavenumbers", "greens_function", "raised_cosine", "anti_aliasing_weights",
    "transfer_function", "shift_lateral", "lateral_table", "lateral_offsets",
    "face_weights", "lens_thickness", "face_symmetric",
    "qpw_delays", "quantize_delays", "incident_field",
    "forward_quick_cpu", "adjoint_quick_cpu", "observation_layout",
    "T_CLK", "EPS",
]

# clock period used to quantise transmit delays (+scattering/+sequences/+setups/setup.m:22)
T_CLK = 1.0 / 80e6
# MATLAB eps used by the occupancy test (+scattering/operator_born.m:361)
EPS = float(np.finfo(np.float64).eps)


@dataclasses.dataclass(frozen=True)
class Absorption:
    """Absorption model of the homogeneous fluid.

    ``kind == "none"``: lossless, ``k = 2*pi*f/c`` (``absorption_models/none.m:83``).
    ``kind == "time_causal"``: power law with optional causal dispersion
    (``absorption_models/time_causal.m:82-83``, ``:118-141``).  ``constant_db``
    is in dB/cm, ``slope_db`` in dB/(MHz^y cm).
    """

    kind: str = "none"
    c: float = 1500.0
    constant_db: float = 0.0
    slope_db: float = 0.0
    exponent: float = 1.0
    f_ref: float = 4e6
    dispersion: bool = True


@dataclasses.dataclass(frozen=True)
class Setup:
    """Discretised pulse-echo setup: planar array + FOV grid + fluid.

    ``n_points_axis`` / ``delta_axis`` list the lateral axes then the axial
    axis.  ``n_elements_axis`` / ``pitch_axis`` / ``width_axis`` /
    ``n_face_axis`` list the lateral axes of the array.
    """

    n_points_axis: tuple
    delta_axis: tuple
    z_start: float
    n_elements_axis: tuple
    pitch_axis: tuple
    width_axis: tuple
    n_face_axis: tuple
    absorption: Absorption = Absorption()
    aa_tx_beta: Optional[float] = 0.5  # raised-cosine roll-off; None = filter off
    aa_rx_beta: Optional[float] = 0.5
    # face weights (face.m:234-285): apodization at the face points (first axis fastest; None =
    # uniform), the lens's axial focus per face axis (empty / 0 / inf = none) and its sound speed
    face_apodization: Optional[tuple] = None
    lens_focus_axis: tuple = ()
    lens_c: float = 1540.0

    # ---- derived quantities -------------------------------------------------
    @property
    def n_dims(self) -> int:
        return len(self.n_points_axis)

    @property
    def n_lat(self) -> int:
        return self.n_dims - 1

    @property
    def n_points(self) -> int:
        return int(np.prod(self.n_points_axis))

    @property
    def n_elements(self) -> int:
        return int(np.prod(self.n_elements_axis))

    @property
    def ppp_axis(self) -> tuple:
        """Grid points per element pitch (``setup.m:1176-1178``); must be integers."""
        out = []
        for p, d in zip(self.pitch_axis, self.delta_axis[: self.n_lat]):
            r = p / d
            if abs(r - round(r)) > 1e-9 * max(1.0, abs(r)):
                raise ValueError("pitch is not an integer multiple of the lateral grid spacing")
            out.append(int(round(r)))
        return tuple(out)

    @property
    def cell_volume(self) -> float:
        """Volume element of the FOV grid (delta_V, ``setup.m:753``)."""
        return float(np.prod(self.delta_axis))

    def axis_positions(self):
        """Per-axis grid coordinates (lateral centred, axial from z_start)."""
        axes = []
        for d in range(self.n_lat):
            n, h = self.n_points_axis[d], self.delta_axis[d]
            axes.append((np.arange(n) - (n - 1) / 2.0) * h)
        n, h = self.n_points_axis[-1], self.delta_axis[-1]
        axes.append(self.z_start + (np.arange(n) + 0.5) * h)
        return axes

    def positions(self) -> np.ndarray:
        """(P, n_dims) grid positions in column-major order."""
        axes = self.axis_positions()
        mesh = np.meshgrid(*axes, indexing="ij")
        return np.stack([m.reshape(-1, order="F") for m in mesh], axis=1)

    def element_centers(self) -> np.ndarray:
        """(E, n_dims) element centroids on the plane z = 0."""
        axes = [(np.arange(n) - (n - 1) / 2.0) * p for n, p in zip(self.n_elements_axis, self.pitch_axis)]
        mesh = np.meshgrid(*axes, indexing="ij")
        lat = np.stack([m.reshape(-1, order="F") for m in mesh], axis=1)
        return np.concatenate([lat, np.zeros((lat.shape[0], 1))], axis=1)

    def face_points(self, e: int):
        """Quadrature points and cell size of element ``e``'s vibrating face.

        Uniform grid of ``n_face_axis`` cells over the face, points at cell
        centres (``face.m:184-229`` + ``orthotope.m:140-146``); the cell size
        is the face grid's ``cell_ref.volume`` used in ``setup.m:1270``.
        """
        ctr = self.element_centers()[e]
        axes, dA = [], 1.0
        for d in range(self.n_lat):
            q, w = self.n_face_axis[d], self.width_axis[d]
            axes.append(ctr[d] + (np.arange(q) - (q - 1) / 2.0) * (w / q))
            dA *= w / q
        mesh = np.meshgrid(*axes, indexing="ij")
        lat = np.stack([m.reshape(-1, order="F") for m in mesh], axis=1)
        pts = np.concatenate([lat, np.zeros((lat.shape[0], 1))], axis=1)
        return pts, dA


# --------------------------------------------------------------------------
# physics
# --------------------------------------------------------------------------
def wavenumbers(setup: Setup, f: np.ndarray) -> np.ndarray:
    """Complex wavenumbers k~(f).

    ``none``: ``absorption_models/none.m:83``.
    ``time_causal``: ``absorption_models/time_causal.m:82-83`` (alpha_0, alpha_1
    from dB), ``:118`` (reference wavenumber), ``:121`` (imaginary part),
    ``:124-136`` (dispersion), ``:145-147`` (zero frequency).
    """
    f = np.asarray(f, dtype=np.float64)
    a = setup.absorption
    if a.kind == "none":
        return (2.0 * np.pi * f / a.c).astype(np.complex128)
    if a.kind != "time_causal":
        raise ValueError(f"unknown absorption model {a.kind}")
    alpha_0 = a.constant_db * math.log(10) / (20 * 0.01)
    alpha_1 = a.slope_db * math.log(10) / (20 * 0.01 * (1e6 ** a.exponent))
    k_ref = 2.0 * np.pi * f / a.c
    k_imag = -alpha_0 - alpha_1 * np.abs(f) ** a.exponent
    if a.dispersion:
        y = a.exponent
        if (y % 2 == 0) or (math.floor(y) != y):
            k_real = k_ref + alpha_1 * math.tan(y * np.pi / 2) * f * (np.abs(f) ** (y - 1) - abs(a.f_ref) ** (y - 1))
        else:
            with np.errstate(divide="ignore"):
                k_real = k_ref - 2 * alpha_1 * f ** y * np.log(np.abs(f / a.f_ref)) / np.pi
    else:
        k_real = k_ref
    k_real = np.where(np.abs(f) < EPS, 0.0, k_real)
    return k_real + 1j * k_imag


def greens_function(n_dims: int, k: np.ndarray, D: np.ndarray) -> np.ndarray:
    """Free-space Green's function (``+processing/greens_function.m:88``, ``:103``).

    2D: ``0.25j * H0^(2)(k D)``; 3D: ``-exp(-j k D) / (4 pi D)``.  ``k`` and
    ``D`` broadcast.
    """
    kD = k * D
    if n_dims == 2:
        return 0.25j * hankel2(0, kD)
    if n_dims == 3:
        return -np.exp(-1j * kD) / (4.0 * np.pi * D)
    raise ValueError("n_dims must be 2 or 3")


def raised_cosine(flags: np.ndarray, beta: float) -> np.ndarray:
    """Raised-cosine window of the local phase shift per pitch.

    ``+scattering/+anti_aliasing_filters/raised_cosine.m:106-119``: 1 for
    flag <= pi(1-beta), 0.5(1+cos(pi (flag-lb)/(pi-lb))) in the taper, 0 for
    flag >= pi.  The product over lateral axes is taken by the caller.
    """
    lb = np.pi * (1.0 - beta)
    ub = np.pi
    out = np.where(flags <= lb, 1.0, 0.0)
    taper = (flags > lb) & (flags < ub)
    out = np.where(taper, 0.5 * (1.0 + np.cos(np.pi * (flags - lb) / (ub - lb))), out)
    return out


def anti_aliasing_weights(setup: Setup, k: np.ndarray, lateral_diff: np.ndarray, dist: np.ndarray,
                          beta: Optional[float]) -> np.ndarray:
    """Spatial anti-aliasing filter applied to a transfer function.

    ``on.m:64-70`` with flags from ``setup.m:916-1032``: flag_d =
    Re(k~) * pitch_d * |e_d| where e is the unit vector from the element
    centroid to the grid point (``setup.m:996-1017``), only over lateral axes
    with more than one element (``setup.m:1000-1002``).

    ``lateral_diff``: (..., n_lat) lateral components of r_p - r_e;
    ``dist``: (...) |r_p - r_e|; ``k``: (F,).  Returns (F, ...).
    """
    shape = (len(k),) + dist.shape
    if beta is None:
        return np.ones(shape)
    w = np.ones(shape)
    for d in range(setup.n_lat):
        if setup.n_elements_axis[d] <= 1:
            continue
        e_abs = np.abs(lateral_diff[..., d]) / dist
        flags = np.real(k).reshape((-1,) + (1,) * dist.ndim) * setup.pitch_axis[d] * e_abs[None]
        w = w * raised_cosine(flags, beta)
    return w


def lens_thickness(setup: Setup) -> np.ndarray:
    """Lens thickness at each face point (``thickness/focus_axial.m``), first axis fastest.

    At the normalised position ``rho = 2 (r_q - r_c) / width`` of a face point
    (``face.m:210-217``), ``t = sum over the focused axes of (sqrt(1 + F^2) -
    sqrt(rho^2 + F^2)) * width / 2`` with ``F = 2 * focus / width``; an axis whose focus is
    infinite (or 0 / absent here) adds nothing.
    """
    fp, _ = setup.face_points(0)
    ctr = setup.element_centers()[0]
    t = np.zeros(fp.shape[0])
    for d in range(setup.n_lat):
        focus = setup.lens_focus_axis[d] if d < len(setup.lens_focus_axis) else 0.0
        if not (np.isfinite(focus) and focus > 0.0):
            continue
        w = setup.width_axis[d]
        rho = 2.0 * (fp[:, d] - ctr[d]) / w
        Fn = 2.0 * focus / w
        t += (np.sqrt(1.0 + Fn ** 2) - np.sqrt(rho ** 2 + Fn ** 2)) * w / 2.0
    return t


def face_weights(setup: Setup, f: np.ndarray) -> np.ndarray:
    """Complex face weights ``(F, Q)``: ``a_q exp(-1j k_lens(f) t_q)``
    (``face.m:359-376`` ``compute_weights_scalar``) with the lens lossless,
    ``k_lens = 2 pi f / c_lens`` (the absorption model ``none`` of ``lens.m``)."""
    Q = int(np.prod([max(1, n) for n in setup.n_face_axis[: setup.n_lat]]))
    a = np.ones(Q) if setup.face_apodization is None else np.asarray(setup.face_apodization, dtype=np.float64)
    k_lens = 2.0 * np.pi * np.asarray(f, dtype=np.float64) / setup.lens_c
    return a[None, :] * np.exp(-1j * k_lens[:, None] * lens_thickness(setup)[None, :])


def face_symmetric(setup: Setup) -> bool:
    """True when the face weights are even in every face axis (the symmetric-grid
    representation ``h_ref`` + ``indices_grid_FOV_shift`` mirrors the reference element's
    transfer function, which needs a face symmetric about its centroid)."""
    if setup.face_apodization is None:
        return True
    q = tuple(max(1, n) for n in setup.n_face_axis[: setup.n_lat])
    a = np.asarray(setup.face_apodization, dtype=np.float64).reshape(q, order="F")
    return all(np.allclose(a, np.flip(a, axis=d), rtol=0, atol=0) for d in range(a.ndim))


def transfer_function(setup: Setup, f: np.ndarray, e: int, beta: Optional[float],
                      points: Optional[np.ndarray] = None) -> np.ndarray:
    """Spatial transfer function of element ``e`` on the FOV grid, (F, P).

    ``setup.m:1216-1281`` (``transfer_function_scalar``):
    ``h = -2 * dA * sum_q w_q(f) G(k~ |r_q - r_p|)`` with the face weights of
    :func:`face_weights` (``setup.m:1241``, applied at ``:1266``), followed by the
    anti-aliasing filter (``setup.m:894-897`` -> ``on.m:64-70``).  ``points``
    optionally restricts the evaluation to a subset of grid indices.
    """
    k = wavenumbers(setup, f)
    pos = setup.positions()
    if points is not None:
        pos = pos[points]
    fp, dA = setup.face_points(e)
    wq = face_weights(setup, f)
    h = np.zeros((len(f), pos.shape[0]), dtype=np.complex128)
    for q in range(fp.shape[0]):
        D = np.linalg.norm(pos - fp[q][None, :], axis=1)
        h -= 2.0 * dA * wq[:, q][:, None] * greens_function(setup.n_dims, k[:, None], D[None, :])
    ctr = setup.element_centers()[e]
    diff = pos - ctr[None, :]
    dist = np.linalg.norm(diff, axis=1)
    h *= anti_aliasing_weights(setup, k, diff[:, : setup.n_lat], dist, beta)
    return h


def shift_lateral(setup: Setup):
    """Index map ``indices_grid_FOV_shift`` of the symmetric-grid setup.

    Restates ``setup_grid_symmetric.m:175-232``: shift each grid point's
    lateral subscripts by ``(e_d - 1) * ppp_d`` (``:184``, ``:196``), mirror
    subscripts <= 0 about ``offset_d = N_d - (E_d - 1) ppp_d + 1``
    (``:199-228``, ``:222``, ``:226``), convert to a 1-based linear index.

    Returns ``(shift, valid)``: shift is (P, E) int64 of 1-based indices into
    the reference element's transfer function; valid is False when any index
    falls outside the grid (the reference would then fail with an indexing
    error; see ``setup.m:1162-1187`` where the range check is a TODO).
    """
    nl = setup.n_lat
    N = np.array(setup.n_points_axis)
    ppp = np.array(setup.ppp_axis)
    Eax = np.array(setup.n_elements_axis)
    # 1-based subscripts of all grid points, column-major
    subs = np.stack(np.unravel_index(np.arange(setup.n_points), tuple(N), order="F"), axis=1) + 1
    esubs = np.stack(np.unravel_index(np.arange(setup.n_elements), tuple(Eax), order="F"), axis=1) + 1
    # one grid axis at a time, broadcast over (points, elements)
    lin = np.zeros((setup.n_points, setup.n_elements), dtype=np.int64)
    valid = True
    stride = 1
    for d in range(setup.n_dims):
        sd = subs[:, d].astype(np.int64)[:, None]
        if d < nl:
            sd = sd - (esubs[None, :, d].astype(np.int64) - 1) * ppp[d]
            offset = N[d] - (Eax[d] - 1) * ppp[d] + 1
            sd = np.where(sd <= 0, offset - sd, sd)
        valid = valid and bool(np.all((sd >= 1) & (sd <= N[d])))
        lin += (np.clip(sd, 1, N[d]) - 1) * stride
        stride *= int(N[d])
    return lin + 1, valid


# --------------------------------------------------------------------------
# lateral-offset table (the layout the CUDA library consumes)
# --------------------------------------------------------------------------
def lateral_offsets(setup: Setup):
    """Per lateral axis: number of signed offsets and their positions.

    On the symmetric grid the transfer function of element ``e`` at grid
    point ``p`` depends only on the signed lateral offset ``i_d - e_d*ppp_d``
    and the axial index.  The offset index ``o_d = i_d - e_d*ppp_d +
    (E_d-1)*ppp_d`` runs over ``[0, N_d + (E_d-1)*ppp_d)``; its lateral
    distance from the element centroid is
    ``(o_d - ((E_d-1)*ppp_d + N_d - 1)/2) * delta_d``.
    """
    out = []
    for d in range(setup.n_lat):
        n_o = setup.n_points_axis[d] + (setup.n_elements_axis[d] - 1) * setup.ppp_axis[d]
        pos = (np.arange(n_o) - (n_o - 1) / 2.0) * setup.delta_axis[d]
        out.append((n_o, pos))
    return out


def lateral_table(setup: Setup, f: np.ndarray, beta: Optional[float]) -> np.ndarray:
    """Transfer-function table indexed by (f, z, [o_y,] o_x).

    Same physics as :func:`transfer_function` (``setup.m:1216-1281`` +
    ``on.m:64-70``), evaluated once per distinct (lateral offset, depth)
    instead of once per (element, point).  Shape ``(F, Nz, No_x)`` in 2D,
    ``(F, Nz, No_y, No_x)`` in 3D.
    """
    k = wavenumbers(setup, f)
    offs = lateral_offsets(setup)
    z = setup.axis_positions()[-1]
    # element-0-relative face offsets; the weights are the same on every element
    fp, dA = setup.face_points(0)
    fp = fp - setup.element_centers()[0][None, :]
    wq = face_weights(setup, f)
    if setup.n_dims == 2:
        Z, X = np.meshgrid(z, offs[0][1], indexing="ij")  # (Nz, No_x)
        lat = X[..., None]
    else:
        Z, Y, X = np.meshgrid(z, offs[1][1], offs[0][1], indexing="ij")  # (Nz, No_y, No_x)
        lat = np.stack([X, Y], axis=-1)
    T = np.zeros((len(f),) + Z.shape, dtype=np.complex128)
    for q in range(fp.shape[0]):
        diff_sq = (Z - fp[q, -1]) ** 2
        for d in range(setup.n_lat):
            diff_sq = diff_sq + (lat[..., d] - fp[q, d]) ** 2
        D = np.sqrt(diff_sq)
        T -= 2.0 * dA * wq[:, q].reshape((-1,) + (1,) * Z.ndim) * greens_function(
            setup.n_dims, k.reshape((-1,) + (1,) * Z.ndim), D[None])
    dist = np.sqrt(Z ** 2 + np.sum(lat ** 2, axis=-1))
    T *= anti_aliasing_weights(setup, k, lat, dist, beta)
    return T


# --------------------------------------------------------------------------
# incident waves
# --------------------------------------------------------------------------
def qpw_delays(setup: Setup, e_theta: Sequence[float]) -> np.ndarray:
    """Quasi-plane-wave transmit delays (``+syntheses/+deterministic/qpw.m:96-97``).

    ``tau_e = <x_e, e_theta_lat> / c``, shifted to a zero minimum.
    ``e_theta`` lists the lateral components of the propagation direction.
    """
    ctr = setup.element_centers()[:, : setup.n_lat]
    tau = ctr @ np.asarray(e_theta, dtype=np.float64)[: setup.n_lat] / setup.absorption.c
    return tau - tau.min()


def quantize_delays(tau: np.ndarray) -> np.ndarray:
    """Round delays to the transmit clock (``setup.m:625``)."""
    return np.round(tau / T_CLK) * T_CLK


def incident_field(setup: Setup, f: np.ndarray, v_d: np.ndarray,
                   h_tx: Callable[[int], np.ndarray]) -> np.ndarray:
    """Incident pressure ``p_in(f, p) = sum_e h_tx_e(f, p) v_d(f, e)``.

    ``+scattering/+sequences/sequence.m:813-844`` (symmetric grid) and
    ``setup.m:1312-1325`` (arbitrary grid): both sum the element transfer
    functions (with the transmit anti-aliasing filter) weighted by the
    normal-velocity spectra ``v_d = excitation * impulse response * delay
    phasor`` (``tx.m:284``, ``setup.m:625-635``).  ``h_tx(e)`` returns (F, P).
    """
    p = np.zeros((len(f), setup.n_points), dtype=np.complex128)
    for e in range(setup.n_elements):
        if np.any(v_d[:, e] != 0):
            p += h_tx(e) * v_d[:, e][:, None]
    return p


# --------------------------------------------------------------------------
# operator tables and the reference's CPU operator
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Mix:
    """One mixed voltage signal of a pulse-echo measurement.

    ``f_idx``: 0-based map of the mix's frequencies to the measurement's
    unique frequencies (``settings(m).indices_f_to_unique{mix}``,
    ``setting.m:268``).  ``active``: 0-based indices of the active elements
    (``rx(mix).indices_active``).  ``pref``: (F_mix, n_active) prefactors
    ``-dV k~^2 * R`` (``sequence.m:590-634``, ``setup.m:759``).
    """

    f_idx: np.ndarray
    active: np.ndarray
    pref: np.ndarray


@dataclasses.dataclass
class Measurement:
    """One sequential pulse-echo measurement (incident wave).

    ``f_idx``: 0-based map of its unique frequencies to the global unique
    frequencies (``sequence.indices_f_to_unique{m}``, ``sequence.m:502``).
    ``p_incident``: (F_meas, P) incident field.
    """

    f_idx: np.ndarray
    p_incident: np.ndarray
    mixes: list


@dataclasses.dataclass
class OperatorTables:
    """Everything ``combined_quick_gpu`` reads from ``operator_born``.

    ``h_ref`` (F_u, P) and ``shift`` (P, E, 1-based) form the symmetric-grid
    representation (``sequence.h_ref``, ``setup.indices_grid_FOV_shift``).
    When the symmetric map is out of range, ``h_element(e)`` gives element
    ``e``'s transfer function at the global frequencies instead (the
    reference's arbitrary-grid branch, ``operator_born.m:437-444``).
    """

    setup: Setup
    f_unique: np.ndarray
    measurements: list
    h_ref: Optional[np.ndarray] = None
    shift: Optional[np.ndarray] = None
    h_element: Optional[Callable[[int], np.ndarray]] = None

    @property
    def n_observations(self) -> int:
        return int(sum(len(m.f_idx) for meas in self.measurements for m in meas.mixes))

    def _h_rx(self, e: int, f_glob: np.ndarray, points: np.ndarray) -> np.ndarray:
        if self.h_ref is not None:
            # operator_born.m:421-431: gather the shifted reference transfer function
            idx = self.shift[points, e] - 1
            return self.h_ref[f_glob][:, idx]
        return self.h_element(e)[f_glob][:, points]


def observation_layout(op: OperatorTables):
    """Row offsets of each (measurement, mix) block in the stacked output.

    Rows are concatenated over measurements, then mixes, then frequencies
    (``operator_born.m:459-463``; ``combined_quick_gpu.cu:978``).
    """
    rows, r = [], 0
    for w, meas in enumerate(op.measurements):
        for m, mix in enumerate(meas.mixes):
            rows.append((w, m, r, len(mix.f_idx)))
            r += len(mix.f_idx)
    return rows, r


def forward_quick_cpu(op: OperatorTables, gamma: np.ndarray) -> np.ndarray:
    """Forward Born operator, restating ``operator_born.m:332-470``.

    Occupied points ``sum|gamma| > eps`` (``:361``); per measurement, mix and
    active element: gather the element's transfer function at the mix's
    frequencies (``:421-444``), ``Phi = h .* p_in .* pref`` (``:451``) and
    ``u += Phi * gamma(occ, :)`` (``:452``).  Frequencies follow the explicit
    index maps in every case, as ``combined_quick_gpu.cu:329-333`` does (the
    MATLAB path skips the map when a mix has as many frequencies as the
    global axis, ``:425``; for the identity maps used here both agree).
    """
    gamma = np.asarray(gamma)
    if gamma.ndim == 1:
        gamma = gamma[:, None]
    occ = np.nonzero(np.sum(np.abs(gamma), axis=1) > EPS)[0]
    B = gamma.shape[1]
    blocks = []
    g_occ = gamma[occ].astype(np.complex128)
    for meas in op.measurements:
        p_occ = meas.p_incident[:, occ]
        for mix in meas.mixes:
            f_glob = meas.f_idx[mix.f_idx]
            p_act = p_occ[mix.f_idx]
            u_mix = np.zeros((len(mix.f_idx), B), dtype=np.complex128)
            if len(occ):
                for a, e in enumerate(mix.active):
                    h_rx = op._h_rx(int(e), f_glob, occ)
                    Phi = h_rx * p_act * mix.pref[:, a][:, None]
                    u_mix += Phi @ g_occ
            blocks.append(u_mix)
    return np.concatenate(blocks, axis=0)


def adjoint_quick_cpu(op: OperatorTables, u: np.ndarray) -> np.ndarray:
    """Adjoint Born operator, restating ``operator_born.m:480-596``.

    ``u`` is split by measurement and mix (``:511-533``); per active element
    ``gamma_hat += Phi' * u_mix`` with ``Phi' `` the conjugate transpose
    (``:583-584``).
    """
    u = np.asarray(u)
    if u.ndim == 1:
        u = u[:, None]
    P = op.setup.n_points
    B = u.shape[1]
    gamma_hat = np.zeros((P, B), dtype=np.complex128)
    allp = np.arange(P)
    r = 0
    for meas in op.measurements:
        for mix in meas.mixes:
            n = len(mix.f_idx)
            u_mix = u[r:r + n].astype(np.complex128)
            r += n
            f_glob = meas.f_idx[mix.f_idx]
            p_act = meas.p_incident[mix.f_idx]
            for a, e in enumerate(mix.active):
                h_rx = op._h_rx(int(e), f_glob, allp)
                Phi = h_rx * p_act * mix.pref[:, a][:, None]
                gamma_hat += Phi.conj().T @ u_mix
    return gamma_hat


def energy_rx_cpu(op: OperatorTables) -> np.ndarray:
    """Received energies in the canonical basis, restating ``energy_rx_canonical``
    (``operator_born.m:718-859``): per measurement and mix, the mixed voltage
    signals of every grid point ``Phi_M = sum_a h_rx * p_in * pref`` (``:773-836``)
    and ``E_M += vecnorm(Phi_M, 2, 1).^2`` (``:853``), i.e. ``E[p] = ||Phi e_p||^2``.
    The reference restricts the method to one selected measurement (``:736-741``);
    the sum here runs over every selected measurement, which is the same column
    norm of the stacked operator.  TGC is the identity (out of scope).
    """
    P = op.setup.n_points
    allp = np.arange(P)
    E = np.zeros(P)
    for meas in op.measurements:
        for mix in meas.mixes:
            f_glob = meas.f_idx[mix.f_idx]
            p_act = meas.p_incident[mix.f_idx]
            Phi_M = np.zeros((len(mix.f_idx), P), dtype=np.complex128)
            for a, e in enumerate(mix.active):
                Phi_M += op._h_rx(int(e), f_glob, allp) * p_act * mix.pref[:, a][:, None]
            E += np.sum(np.abs(Phi_M) ** 2, axis=0)
    return E
