"""CPU checks of the FP64 oracle (no GPU).

The reference is MATLAB-only and pins no numbers on this path, so the oracle
is checked against mathematics and against itself along independent routes:
mpmath Hankel functions, closed-form single-term answers, the reference's own
symmetric-grid index map versus direct per-element evaluation, the
lateral-offset table versus both, exact adjointness, and frozen golden
fixtures.
"""

import numpy as np
import pytest

from oracle import (Absorption, Setup, adjoint_quick_cpu, forward_quick_cpu, greens_function,
                    lateral_table, raised_cosine, shift_lateral, transfer_function, wavenumbers)
from oracle import configs
from tests.golden import make_golden


def test_hankel_against_mpmath():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 30
    # arguments k~*D over the workloads' range: |kD| ~ 10 .. 3000, small absorption
    for kd in [10.3 - 0.01j, 41.9 - 0.2j, 255.5 - 1.1j, 1760.0 - 3.0j, 3000.0 - 0.5j, 12.0 - 0j]:
        ref = complex(mpmath.hankel2(0, mpmath.mpc(kd.real, kd.imag)))
        got = greens_function(2, np.array(kd), np.array(1.0)) / 0.25j
        assert abs(got - ref) <= 1e-12 * abs(ref)


def test_greens_3d_closed_form():
    k, D = 2 * np.pi * 4e6 / 1500.0, 7e-3
    g = greens_function(3, np.array(k), np.array(D))
    assert abs(g - (-np.exp(-1j * k * D) / (4 * np.pi * D))) < 1e-15 * abs(g)


def test_wavenumbers():
    s = Setup((4, 4), (1e-4, 1e-4), 1e-3, (2,), (2e-4,), (1.8e-4,), (1,), Absorption("none", 1540.0))
    f = np.array([1e6, 5e6])
    np.testing.assert_allclose(wavenumbers(s, f), 2 * np.pi * f / 1540.0, rtol=1e-15)
    tc = Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True)
    s2 = Setup((4, 4), (1e-4, 1e-4), 1e-3, (2,), (2e-4,), (1.8e-4,), (1,), tc)
    k = wavenumbers(s2, np.array([4e6, 2e6, 6e6]))
    alpha_1 = 0.5 * np.log(10) / (20 * 0.01 * 1e6)
    # at f_ref the dispersion term vanishes; Im k = -alpha_1 * f (y = 1)
    assert abs(k[0].real - 2 * np.pi * 4e6 / 1500.0) < 1e-9
    np.testing.assert_allclose(-k.imag, alpha_1 * np.array([4e6, 2e6, 6e6]), rtol=1e-14)
    # causal dispersion (y odd): phase velocity rises with frequency
    c_phase = 2 * np.pi * np.array([2e6, 6e6]) / k[1:].real
    assert c_phase[0] < 1500.0 < c_phase[1]


def test_raised_cosine_window():
    beta = 0.5
    lb = np.pi * (1 - beta)
    w = raised_cosine(np.array([0.0, lb, 0.5 * (lb + np.pi), np.pi, 4.0]), beta)
    np.testing.assert_allclose(w, [1.0, 1.0, 0.5, 0.0, 0.0], atol=1e-15)


def test_single_term_known_answer():
    """One element, one point, one frequency: u = h * p_in * pref * gamma in closed form."""
    s = Setup((1, 1), (1e-4, 1e-4), 5e-3, (1,), (1e-4,), (0.9e-4,), (1,), Absorption("none", 1500.0),
              aa_tx_beta=None, aa_rx_beta=None)
    f = np.array([3e6])
    k = 2 * np.pi * 3e6 / 1500.0
    D = 5e-3 + 0.5e-4
    from scipy.special import hankel2
    h_expected = -2 * 0.9e-4 * 0.25j * hankel2(0, k * D)
    h = transfer_function(s, f, 0, None)
    assert abs(h[0, 0] - h_expected) < 1e-15 * abs(h_expected)
    from oracle import Measurement, Mix, OperatorTables
    pref = -(1e-4 * 1e-4) * k ** 2
    op = OperatorTables(setup=s, f_unique=f, h_ref=h, shift=np.array([[1]]),
                        measurements=[Measurement(np.array([0]), np.array([[2.0 - 1j]]),
                                                  [Mix(np.array([0]), np.array([0]), np.array([[pref]]))])])
    u = forward_quick_cpu(op, np.array([[3.0]]))
    assert abs(u[0, 0] - h_expected * (2.0 - 1j) * pref * 3.0) < 1e-14 * abs(u[0, 0])


@pytest.mark.parametrize("name,valid", [("c0", False), ("c1", True), ("c2", True), ("c3", True)])
def test_symmetric_map_validity(name, valid):
    """The reference's mirrored shift is in range only when the FOV spans the array."""
    _, ok = shift_lateral(configs.small_config(name).setup)
    assert ok == valid
    # the full-size 2D plain workload (256-point FOV, 508-point array span) is out of range too
    if name == "c0":
        _, ok_full = shift_lateral(configs.config("c0").setup)
        assert not ok_full


@pytest.mark.parametrize("name", ["c1", "c3"])
def test_symmetric_map_and_lateral_table_equal_direct_evaluation(name):
    cfg = configs.small_config(name)
    s = cfg.setup
    f = cfg.f[:3]
    shift, ok = shift_lateral(s)
    assert ok
    h_ref = transfer_function(s, f, 0, s.aa_rx_beta)
    T = lateral_table(s, f, s.aa_rx_beta)
    for e in range(0, s.n_elements, max(1, s.n_elements // 5)):
        h_e = transfer_function(s, f, e, s.aa_rx_beta)
        scale = np.max(np.abs(h_e))
        assert np.max(np.abs(h_ref[:, shift[:, e] - 1] - h_e)) <= 1e-12 * scale
        assert np.max(np.abs(configs.element_from_table(s, T, e) - h_e)) <= 1e-12 * scale


@pytest.mark.parametrize("name", ["c0", "c1", "c2", "ragged", "c3"])
def test_oracle_adjointness(name):
    b = configs.build(configs.small_config(name))
    rng = np.random.default_rng(3)
    x = configs.make_gamma(b.cfg, complex_values=True)
    u = forward_quick_cpu(b.op, x)
    y = rng.standard_normal(u.shape) + 1j * rng.standard_normal(u.shape)
    lhs = np.vdot(y, u)
    rhs = np.vdot(adjoint_quick_cpu(b.op, y), x)
    assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(u) * np.linalg.norm(y)


def test_occupancy_does_not_change_result():
    """Restricting the forward sum to occupied points (operator_born.m:361) is exact."""
    b = configs.build(configs.small_config("c1"))
    g = configs.make_gamma(b.cfg)
    u_sparse = forward_quick_cpu(b.op, g)
    # the same sum over every point: add an all-ones column, subtract its contribution
    g2 = np.concatenate([g, np.ones_like(g)], axis=1)
    u_dense = forward_quick_cpu(b.op, g2)[:, :1]
    np.testing.assert_allclose(u_dense, u_sparse, rtol=1e-12, atol=1e-12 * np.max(np.abs(u_sparse)))


def test_element_path_matches_symmetric_path():
    """Arbitrary-grid branch (direct element transfer functions) equals the symmetric gather."""
    cfg = configs.small_config("c1")
    b_sym = configs.build(cfg)
    import dataclasses
    b_dir = configs.build(cfg, direct_elements=True)
    op_dir = dataclasses.replace(b_dir.op, h_ref=None, shift=None,
                                 h_element=lambda e: transfer_function(cfg.setup, cfg.f, e, cfg.setup.aa_rx_beta))
    g = configs.make_gamma(cfg)
    u1 = forward_quick_cpu(b_sym.op, g)
    u2 = forward_quick_cpu(op_dir, g)
    assert np.linalg.norm(u1 - u2) <= 1e-12 * np.linalg.norm(u1)


def test_golden_fixture_reproduced():
    gold = np.load(make_golden.OUT)
    now = make_golden.generate()
    for k in gold.files:
        ref = gold[k]
        np.testing.assert_allclose(now[k], ref, rtol=1e-12, atol=1e-13 * max(1e-300, float(np.max(np.abs(ref)))),
                                   err_msg=k)


@pytest.mark.parametrize("wname,cname", [("2d-plain", "c0"), ("2d-gradient", "c1"), ("2d-batched", "c2"),
                                         ("3d", "c3")])
def test_benchmark_workloads_match_oracle_configs(wname, cname):
    """The benchmark's synthetic inputs are the oracle's workloads, value for value."""
    from comp_ui_toolbox_gb300.workloads import workload
    w = workload(wname)
    c = configs.config(cname)
    s = c.setup
    assert w.n_points_axis == s.n_points_axis and w.n_elements_axis == s.n_elements_axis
    np.testing.assert_allclose(w.delta_axis, s.delta_axis, rtol=0)
    np.testing.assert_allclose(w.pitch_axis, s.pitch_axis, rtol=0)
    np.testing.assert_allclose(w.width_axis, s.width_axis, rtol=0)
    assert w.z_start == s.z_start and w.n_face_axis == s.n_face_axis
    assert w.absorption["kind"] == s.absorption.kind and w.absorption["c"] == s.absorption.c
    if s.absorption.kind == "time_causal":
        assert w.absorption["slope_db"] == s.absorption.slope_db and w.absorption["f_ref"] == s.absorption.f_ref
    np.testing.assert_array_equal(w.f, c.f)
    assert len(w.waves) == len(c.waves)
    for ww, cw in zip(w.waves, c.waves):
        np.testing.assert_allclose(w.wave_vd(ww), configs.wave_vd(c, cw, c.f), rtol=1e-15, atol=1e-15)
    np.testing.assert_array_equal(w.mix_weights(), configs.mix_weights(c))
    assert w.n_objects == c.n_objects and w.density == c.density and w.seed == c.seed
    np.testing.assert_array_equal(w.gamma(n_objects=1), configs.make_gamma(c, n_objects=1))


def test_energy_rx_restatement_equals_column_norms():
    """The energy_rx restatement equals ||Phi e_p||^2 taken from explicit columns of the forward."""
    from oracle.born_oracle import energy_rx_cpu
    b = configs.build(configs.small_config("c2"))
    E = energy_rx_cpu(b.op)
    P = b.cfg.setup.n_points
    for p in np.random.default_rng(0).choice(P, 4, replace=False):
        e = np.zeros((P, 1))
        e[p] = 1.0
        col = forward_quick_cpu(b.op, e)
        assert abs(E[p] - np.sum(np.abs(col) ** 2)) <= 1e-12 * E[p]
