"""Bridges between the oracle's tables and the library's host mirror (tests only)."""

from __future__ import annotations

import numpy as np

from oracle import configs


def rel_l2(x, ref) -> float:
    # in double precision: the squares of FP32 values such as received energies (~1e-26) underflow
    x = np.asarray(x).astype(np.complex128)
    ref = np.asarray(ref).astype(np.complex128)
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


def make_operator(built: configs.BuiltOperator, form: str = "lateral", max_objects: int = 1, device: int = 0):
    """OperatorBorn over the same tables the oracle uses.

    ``form='lateral'`` passes the lateral-offset table; ``form='reference'``
    passes the reference's own ``h_ref`` + ``indices_grid_FOV_shift``.
    """
    from comp_ui_toolbox_gb300 import OperatorBorn

    s = built.cfg.setup
    kw = dict(n_points_axis=s.n_points_axis, n_elements_axis=s.n_elements_axis,
              n_points_per_pitch=s.ppp_axis, n_f_unique=len(built.op.f_unique),
              measurements=built.op.measurements, device=device, max_objects=max_objects)
    if form == "lateral":
        return OperatorBorn(h_lateral=built.table_rx, **kw)
    if form == "reference":
        assert built.op.h_ref is not None, "symmetric index map out of range for this setup"
        return OperatorBorn(h_ref=built.op.h_ref, indices_grid_FOV_shift=built.op.shift, **kw)
    raise ValueError(form)


def setup_kwargs(cfg: configs.BornConfig) -> dict:
    """Arguments of OperatorBorn.from_setup describing the same operator as the oracle config."""
    s = cfg.setup
    a = s.absorption
    absorption = dict(kind=a.kind, c=a.c, constant_db=a.constant_db, slope_db=a.slope_db, exponent=a.exponent,
                      f_ref=a.f_ref, dispersion=a.dispersion)
    f = np.asarray(cfg.f, dtype=np.float64)
    waves = []
    for wave in cfg.waves:
        f_idx = np.arange(len(f)) if wave.f_subset is None else np.asarray(wave.f_subset)
        mixes = [dict(f_idx=mf, active=act, response=resp) for mf, act, resp in configs.mix_layout(cfg, len(f_idx))]
        waves.append(dict(f_idx=f_idx, v_d=configs.wave_vd(cfg, wave, f[f_idx]), mixes=mixes))
    nl = s.n_lat
    return dict(n_points_axis=s.n_points_axis, delta_axis=s.delta_axis, z_start=s.z_start,
                n_elements_axis=s.n_elements_axis, pitch_axis=s.pitch_axis[:nl], width_axis=s.width_axis[:nl],
                n_face_axis=s.n_face_axis[:nl], absorption=absorption, f_unique=f, waves=waves,
                aa_tx_beta=s.aa_tx_beta, aa_rx_beta=s.aa_rx_beta, face_apodization=s.face_apodization,
                lens_focus_axis=tuple(s.lens_focus_axis), lens_c=s.lens_c)
