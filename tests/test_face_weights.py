"""Face apodization and lens weights of the setup form (face.m:234-285, setup.m:1241-1269).

The transfer function sums, over the face's quadrature points q,
``w_q(f) G(k~(f), |r - r_q|)`` with ``w_q(f) = a_q exp(-j k_lens(f) t_q)``: ``a_q`` the face's
apodization at the point's normalised position, ``t_q`` the lens thickness of
``thickness/focus_axial.m`` and ``k_lens`` the lossless lens's wavenumber.

CPU: the oracle's restatement (``face_weights`` / ``lens_thickness``) against the closed form
of ``focus_axial.m``, uniform weights that leave the unweighted table unchanged, and the
linearity of the transfer function in the per-point weights.  GPU: plans built from setups with
a non-uniform (Hann) apodization and a focusing lens, against the oracle, 2D and 3D (stored,
streamed and generated tables), relative L2 <= 1e-5.
"""

import dataclasses

import numpy as np
import pytest

from oracle import Absorption, Setup, configs
from oracle.born_oracle import face_weights, lens_thickness, transfer_function

TOL = 1e-5


def hann(n):
    """Hann apodization at the normalised face positions rho = (2q - n + 1) / n: cos^2(pi rho / 2)."""
    rho = (2.0 * np.arange(n) - n + 1.0) / n
    return np.cos(np.pi * rho / 2.0) ** 2


def setup_2d(**kw):
    return Setup(n_points_axis=(40, 12), delta_axis=(1e-4, 1e-4), z_start=2e-3, n_elements_axis=(6,),
                 pitch_axis=(3e-4,), width_axis=(2.7e-4,), n_face_axis=(5,),
                 absorption=Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True), **kw)


def test_uniform_weights_are_ones():
    s = setup_2d()
    assert np.array_equal(face_weights(s, np.array([2e6, 5e6])), np.ones((2, 5)))


def test_lens_thickness_is_the_focus_axial_profile():
    focus = 16e-3
    s = setup_2d(lens_focus_axis=(focus,))
    w = s.width_axis[0]
    rho = (2.0 * np.arange(5) - 5 + 1.0) / 5
    Fn = 2 * focus / w
    expect = (np.sqrt(1 + Fn ** 2) - np.sqrt(rho ** 2 + Fn ** 2)) * w / 2
    assert np.allclose(lens_thickness(s), expect, rtol=1e-14, atol=0)
    assert lens_thickness(s)[2] == pytest.approx((np.sqrt(1 + Fn ** 2) - Fn) * w / 2, rel=1e-14)
    # an unfocused axis (infinite focus) adds nothing
    assert np.array_equal(lens_thickness(setup_2d(lens_focus_axis=(np.inf,))), np.zeros(5))
    f = np.array([3e6])
    wq = face_weights(dataclasses.replace(s, face_apodization=tuple(hann(5))), f)
    assert np.allclose(wq, hann(5)[None] * np.exp(-1j * 2 * np.pi * f[:, None] / 1540.0 * expect[None]), rtol=1e-14)


def test_transfer_function_is_linear_in_the_point_weights():
    """With apodization a, h equals sum_q a_q h(one-hot weight at q)."""
    a = hann(5) + 0.1
    s = setup_2d(face_apodization=tuple(a), lens_focus_axis=(12e-3,))
    f = np.array([2.5e6, 4e6])
    h = transfer_function(s, f, 0, 0.5)
    parts = [transfer_function(dataclasses.replace(s, face_apodization=tuple(np.eye(5)[q])), f, 0, 0.5)
             for q in range(5)]
    assert np.allclose(h, sum(a_q * p for a_q, p in zip(a, parts)), rtol=1e-12, atol=0)


def test_python_descriptor_checks_the_apodization_length():
    from comp_ui_toolbox_gb300 import CuiError
    from comp_ui_toolbox_gb300.born import setup_desc
    from tests.helpers import setup_kwargs
    cfg = configs.BornConfig("fw", setup_2d(), np.linspace(2e6, 4e6, 3), [configs.Wave("qpw", (0.0,))])
    kw = setup_kwargs(cfg)
    kw["face_apodization"] = np.ones(4)
    with pytest.raises(CuiError):
        setup_desc(**kw)


# ---------------------------------------------------------------------------
# GPU: device tables with face weights against the oracle
# ---------------------------------------------------------------------------
def weighted_configs():
    s2 = setup_2d(face_apodization=tuple(hann(5)), lens_focus_axis=(10e-3,), lens_c=1200.0)
    c2 = configs.BornConfig("fw-2d", s2, np.linspace(2e6, 5e6, 6), [configs.Wave("qpw", (8.0,)),
                                                                     configs.Wave("qpw", (-5.0,))], seed=4)
    a3 = np.outer(hann(3), hann(4) + 0.2).reshape(-1, order="F")  # first axis fastest
    s3 = Setup(n_points_axis=(12, 10, 8), delta_axis=(1e-4, 1e-4, 1e-4), z_start=2e-3, n_elements_axis=(3, 3),
               pitch_axis=(3e-4, 3e-4), width_axis=(2.6e-4, 2.4e-4), n_face_axis=(3, 4),
               absorption=Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True),
               face_apodization=tuple(a3), lens_focus_axis=(np.inf, 8e-3))
    c3 = configs.BornConfig("fw-3d", s3, np.linspace(2e6, 4e6, 4), [configs.Wave("qpw", (5.0, 0.0))], seed=5)
    return {"2d": c2, "3d": c3}


@pytest.mark.gpu
@pytest.mark.parametrize("name,storage", [("2d", "stored"), ("3d", "stored"), ("3d", "streamed"), ("3d", "generated")])
def test_setup_form_face_weights_match_oracle(name, storage):
    torch = pytest.importorskip("torch")
    from comp_ui_toolbox_gb300 import OperatorBorn
    from oracle import adjoint_quick_cpu, forward_quick_cpu
    from tests.helpers import rel_l2, setup_kwargs
    cfg = weighted_configs()[name]
    b = configs.build(cfg)
    op = OperatorBorn.from_setup(**setup_kwargs(cfg), max_objects=2, table_storage=storage)
    gamma = configs.make_gamma(cfg, n_objects=2, complex_values=True)
    u = op.forward(torch.from_numpy(gamma.astype(np.complex64)).cuda()).cpu().numpy()
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= TOL
    rng = np.random.default_rng(2)
    y = rng.standard_normal((op.n_observations, 2)) + 1j * rng.standard_normal((op.n_observations, 2))
    g = op.adjoint(torch.from_numpy(y.astype(np.complex64)).cuda()).cpu().numpy()
    assert rel_l2(g, adjoint_quick_cpu(b.op, y)) <= TOL
    # the weights change the operator: the same setup without them is far from it
    plain = dataclasses.replace(cfg, setup=dataclasses.replace(cfg.setup, face_apodization=None, lens_focus_axis=()))
    assert rel_l2(forward_quick_cpu(configs.build(plain).op, gamma), u) > 1e-2
    op.close()
