"""Bridges between the oracle's tables and the library's host mirror (tests only)."""

from __future__ import annotations

import numpy as np

from oracle import configs


def rel_l2(x, ref) -> float:
    x = np.asarray(x)
    ref = np.asarray(ref)
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
