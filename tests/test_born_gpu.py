"""GPU parity tests of the FP32 Born operator against the FP64 oracle.

Every call goes through libcui_born.so's C-ABI (via the ctypes host mirror).
Tolerance: relative L2 error <= 1e-5 against the FP64 oracle for every
output (forward, adjoint, VJP), the bound the operator is specified to.
"""

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, forward_quick_cpu
from oracle import configs
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5          # relative L2 vs FP64 oracle
TOL_DOT = 1e-6      # dot-product (adjointness) test, relative to |Phi x| |y|

CONFIGS = ["c0", "c1", "c2", "ragged", "c3", "five"]
_BUILT = {}


def built(name):
    if name not in _BUILT:
        _BUILT[name] = configs.build(configs.small_config(name))
    return _BUILT[name]


def dev(x):
    return torch.from_numpy(np.asarray(x, dtype=np.complex64)).cuda()


def rand_obs(b, n_cols, seed):
    rng = np.random.default_rng(seed)
    n = b.op.n_observations
    return rng.standard_normal((n, n_cols)) + 1j * rng.standard_normal((n, n_cols))


@pytest.mark.parametrize("name", CONFIGS)
def test_forward_adjoint_match_oracle(name):
    b = built(name)
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    gamma = configs.make_gamma(b.cfg)
    u_ref = forward_quick_cpu(b.op, gamma)
    u = op.forward(dev(gamma)).cpu().numpy()
    assert u.shape == u_ref.shape
    assert rel_l2(u, u_ref) <= TOL
    y = rand_obs(b, B, 7)
    g_ref = adjoint_quick_cpu(b.op, y)
    g = op.adjoint(dev(y)).cpu().numpy()
    assert rel_l2(g, g_ref) <= TOL


@pytest.mark.parametrize("name,B", [("c2", 40), ("ragged", 9)])
def test_batched_mixing_matches_oracle(name, B):
    """Batches of 8 or more objects take the slot-tiled mixing and unmixing (one block per slot
    and 32 objects, the slot's prefactors staged as a dense matrix); 40 objects leave the second
    object block partly filled, and the ragged setup has mixes over frequency subsets.  Forward
    and adjoint per object against the oracle, in FP32 and split-BF16."""
    b = built(name)
    op = make_operator(b, "lateral", max_objects=B)
    gamma = configs.make_gamma(b.cfg, n_objects=B, seed=21)
    u_ref = forward_quick_cpu(b.op, gamma)
    y = rand_obs(b, B, 8)
    g_ref = adjoint_quick_cpu(b.op, y)
    for precision in ("fp32", "bf16x3"):
        op.set_precision(precision)
        u = op.forward(dev(gamma)).cpu().numpy()
        g = op.adjoint(dev(y)).cpu().numpy()
        for k in range(B):
            assert rel_l2(u[:, k], u_ref[:, k]) <= TOL
            assert rel_l2(g[:, k], g_ref[:, k]) <= TOL
    assert op.device_status() == 0


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
@pytest.mark.parametrize("staging", ["direct", "staging"])
def test_host_vjp_matches_device_vjp(precision, staging, monkeypatch):
    """cui_born_vjp_host on 20 objects, through both host paths (direct access to the caller's
    arrays, or pinned staging), against the device VJP of the same objects: the same device
    computation, so equal to rounding of the FP64 <-> FP32 conversions (relative 1e-6), and
    within the operator's bound of the oracle."""
    monkeypatch.setenv("CUI_BORN_HOST_STAGING", "1" if staging == "staging" else "0")
    b = built("c2")
    B = 20
    op = make_operator(b, "lateral", max_objects=B)
    op.set_precision(precision)
    gamma = configs.make_gamma(b.cfg, n_objects=B, seed=31)
    u_meas = rand_obs(b, B, 32)
    grad_d, loss_d = op.vjp(dev(gamma), dev(u_meas))
    grad_d = grad_d.cpu().numpy()
    loss_d = loss_d.cpu().numpy()
    grad_h, loss_h = op.vjp(gamma, u_meas)
    r = forward_quick_cpu(b.op, gamma) - u_meas
    g_ref = adjoint_quick_cpu(b.op, r)
    for k in range(B):
        assert rel_l2(grad_h[:, k], grad_d[:, k]) <= 1e-6
        assert rel_l2(grad_h[:, k], g_ref[:, k]) <= TOL
    np.testing.assert_allclose(loss_h, loss_d, rtol=1e-6)
    assert op.device_status() == 0


def test_host_output_with_8_byte_alignment():
    """The host write-back stores 16 bytes per element when the caller's array is 16-byte aligned
    and 8 bytes at a time otherwise: an output whose base sits 8 bytes off a 16-byte boundary gets
    the same values as an aligned one (direct host path)."""
    b = built("c2")
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    gamma = configs.make_gamma(b.cfg, complex_values=True)
    u = configs.add_noise(forward_quick_cpu(b.op, gamma), 30.0, seed=3)
    g0 = np.asfortranarray(gamma)
    u0 = np.asfortranarray(u)
    grad_a, loss_a = op.vjp(g0, u0)
    nbytes = g0.size * 16
    raw = np.zeros(nbytes + 32, dtype=np.uint8)
    off = (8 - raw.ctypes.data % 16) % 16
    out = raw[off:off + nbytes].view(np.complex128).reshape(g0.shape, order="F")
    assert out.ctypes.data % 16 == 8 and out.flags.f_contiguous
    grad_u, loss_u = op.vjp(g0, u0, out=out)
    assert np.array_equal(out, grad_a)
    assert np.array_equal(loss_u, loss_a)
    # an array that breaks the element type's 8-byte alignment is refused before any launch
    from comp_ui_toolbox_gb300 import CuiError
    off4 = (4 - raw.ctypes.data % 16) % 16
    bad = raw[off4:off4 + nbytes].view(np.complex128).reshape(g0.shape, order="F")
    with pytest.raises(CuiError) as ei:
        op.vjp(g0, u0, out=bad)
    assert ei.value.status == 1
    assert op.device_status() == 0
    op.close()


@pytest.mark.parametrize("name", ["c1", "c2", "ragged", "c3"])
def test_reference_form_matches_lateral_form(name):
    """The reference's h_ref + indices_grid_FOV_shift give the same operator."""
    b = built(name)
    B = b.cfg.n_objects
    op_ref = make_operator(b, "reference", max_objects=B)
    op_lat = make_operator(b, "lateral", max_objects=B)
    gamma = dev(configs.make_gamma(b.cfg, complex_values=True))
    u_ref = op_ref.forward(gamma).cpu().numpy()
    u_lat = op_lat.forward(gamma).cpu().numpy()
    assert rel_l2(u_ref, u_lat) <= 1e-6
    assert rel_l2(u_ref, forward_quick_cpu(b.op, gamma.cpu().numpy().astype(np.complex128))) <= TOL


@pytest.mark.parametrize("name", ["c1", "ragged"])
@pytest.mark.parametrize("staging", ["direct", "staging"])
def test_host_path_matches_oracle(name, staging, monkeypatch):
    """FP64 host buffers in, FP64 out: the MEX gateway's semantics.  Both host paths: kernels that
    read and write the caller's pageable arrays (where the GPU uses the host's page tables) and
    the pinned staging buffers (CUI_BORN_HOST_STAGING=1)."""
    monkeypatch.setenv("CUI_BORN_HOST_STAGING", "1" if staging == "staging" else "0")
    b = built(name)
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    gamma = configs.make_gamma(b.cfg)
    u = op.forward(gamma)
    assert u.dtype == np.complex128
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= TOL
    y = rand_obs(b, B, 3)
    assert rel_l2(op.adjoint(y), adjoint_quick_cpu(b.op, y)) <= TOL
    assert op.combined_scalar(0) == (b.op.n_observations, b.cfg.setup.n_points)


@pytest.mark.parametrize("name", CONFIGS)
def test_dot_product_adjointness(name):
    b = built(name)
    op = make_operator(b, "lateral", max_objects=1)
    rng = np.random.default_rng(11)
    P = b.cfg.setup.n_points
    x = rng.standard_normal(P) + 1j * rng.standard_normal(P)
    y = rand_obs(b, 1, 12)[:, 0]
    Ax = op.forward(dev(x)).cpu().numpy().astype(np.complex128)
    AHy = op.adjoint(dev(y)).cpu().numpy().astype(np.complex128)
    lhs = np.vdot(y, Ax)
    rhs = np.vdot(AHy, x)
    assert abs(lhs - rhs) <= TOL_DOT * np.linalg.norm(Ax) * np.linalg.norm(y)


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_vjp_matches_oracle(name):
    b = built(name)
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    gamma_true = configs.make_gamma(b.cfg)
    u_meas = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 30.0, seed=5)
    rng = np.random.default_rng(21)
    gamma = rng.standard_normal(gamma_true.shape)
    r = forward_quick_cpu(b.op, gamma) - u_meas
    grad_ref = adjoint_quick_cpu(b.op, r)
    loss_ref = 0.5 * np.sum(np.abs(r) ** 2, axis=0)
    grad, loss = op.vjp(dev(gamma), dev(u_meas))
    assert rel_l2(grad.cpu().numpy(), grad_ref) <= TOL
    np.testing.assert_allclose(loss.cpu().numpy(), loss_ref, rtol=TOL)
    grad_h, loss_h = op.vjp(gamma, u_meas)
    assert rel_l2(grad_h, grad_ref) <= TOL
    np.testing.assert_allclose(loss_h, loss_ref, rtol=TOL)


def test_vjp_central_finite_differences():
    """d/dt 0.5||Phi(g + t d) - u||^2 at t=0 equals Re<grad, d> (step 1e-3 relative)."""
    b = built("c1")
    op = make_operator(b, "lateral", max_objects=1)
    rng = np.random.default_rng(31)
    P = b.cfg.setup.n_points
    gamma = rng.standard_normal(P)
    u_meas = configs.add_noise(forward_quick_cpu(b.op, configs.make_gamma(b.cfg))[:, 0], 30.0, seed=2)
    grad, _ = op.vjp(gamma, u_meas)
    d = rng.standard_normal(P)
    h = 1e-3 * np.linalg.norm(gamma) / np.linalg.norm(d)
    _, lp = op.vjp(gamma + h * d, u_meas)
    _, lm = op.vjp(gamma - h * d, u_meas)
    fd = (lp - lm) / (2 * h)
    an = np.real(np.vdot(grad, d))
    assert abs(fd - an) <= 2e-3 * abs(an)


def test_torch_autograd_backward_is_adjoint():
    from comp_ui_toolbox_gb300 import born_forward
    b = built("c1")
    op = make_operator(b, "lateral", max_objects=1)
    rng = np.random.default_rng(41)
    P = b.cfg.setup.n_points
    g = dev(rng.standard_normal(P) + 1j * rng.standard_normal(P)).requires_grad_(True)
    u_meas = dev(rand_obs(b, 1, 42)[:, 0])
    u = born_forward(g, op)
    loss = 0.5 * (u - u_meas).abs().pow(2).sum()
    loss.backward()
    grad_vjp, loss_vjp = op.vjp(g.detach(), u_meas)
    assert rel_l2(g.grad.cpu().numpy(), grad_vjp.cpu().numpy()) <= 1e-6
    assert abs(loss.item() - loss_vjp.item()) <= 1e-5 * loss.item()


def test_deterministic_and_linear():
    b = built("c2")
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    g1 = dev(configs.make_gamma(b.cfg, seed=1))
    g2 = dev(configs.make_gamma(b.cfg, seed=2))
    u1 = op.forward(g1)
    u1b = op.forward(g1)
    assert torch.equal(u1, u1b)                      # bitwise reproducible
    u2 = op.forward(g2)
    u12 = op.forward(g1 + 2.0 * g2)
    assert rel_l2(u12.cpu().numpy(), (u1 + 2.0 * u2).cpu().numpy()) <= 1e-6
    z = op.forward(torch.zeros_like(g1))
    assert torch.count_nonzero(z) == 0


def test_leading_dimension_and_subset_of_columns():
    """Column-major inputs with ld > rows and fewer columns than max_objects."""
    import ctypes as C
    b = built("c2")
    op = make_operator(b, "lateral", max_objects=6)
    P, N = b.cfg.setup.n_points, b.op.n_observations
    gamma = configs.make_gamma(b.cfg)[:, :3]
    ld = P + 5
    buf = torch.zeros((3, ld), dtype=torch.complex64, device="cuda")
    buf[:, :P] = dev(gamma.T)
    ldu = N + 3
    out = torch.full((3, ldu), 7.0 + 0j, dtype=torch.complex64, device="cuda")
    st = op._lib.cui_born_forward(op._plan, buf.data_ptr(), ld, 3, out.data_ptr(), ldu,
                                  torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    u = out[:, :N].cpu().numpy().T
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= TOL
    assert torch.all(out[:, N:] == 7.0)              # padding rows untouched
    del C


def test_errors_are_reported():
    from comp_ui_toolbox_gb300 import CuiError
    b = built("c1")
    op = make_operator(b, "lateral", max_objects=1)
    with pytest.raises(CuiError) as ei:
        op.forward(dev(np.zeros((b.cfg.setup.n_points, 2))))   # more columns than max_objects
    assert ei.value.status == 1
    # symmetric index map out of range (FOV narrower than the array): the reference would fail
    b0 = built("c0")
    with pytest.raises(CuiError) as ei:
        make_operator(configs.BuiltOperator(b0.cfg, _with_map(b0), b0.table_rx, b0.table_tx, False), "reference")
    assert ei.value.status == 2
    # a map that is not the symmetric lateral shift is refused
    b1 = built("c1")
    bad = b1.op.shift.copy()
    bad[0, 3] = bad[1, 3]
    opb = _with_map(b1, bad)
    with pytest.raises(CuiError) as ei:
        make_operator(configs.BuiltOperator(b1.cfg, opb, b1.table_rx, b1.table_tx, True), "reference")
    assert ei.value.status == 2


def _with_map(b, shift=None):
    import dataclasses
    from oracle import shift_lateral, transfer_function
    s = b.cfg.setup
    if shift is None:
        shift, _ = shift_lateral(s)
    h_ref = b.op.h_ref if b.op.h_ref is not None else transfer_function(s, b.op.f_unique, 0, s.aa_rx_beta)
    return dataclasses.replace(b.op, h_ref=h_ref, shift=shift)


def test_native_kernels_launched():
    from comp_ui_toolbox_gb300 import launch_count
    b = built("c1")
    op = make_operator(b, "lateral", max_objects=1)
    n0 = launch_count()
    op.forward(dev(configs.make_gamma(b.cfg)))
    torch.cuda.synchronize()
    assert launch_count() - n0 >= 3


@pytest.mark.parametrize("name", CONFIGS)
def test_setup_form_tables_built_on_device(name):
    """Tables computed on the GPU (FP64 Green's functions, FP32 storage) give the oracle's operator."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from tests.helpers import setup_kwargs
    b = built(name)
    B = b.cfg.n_objects
    op = OperatorBorn.from_setup(**setup_kwargs(b.cfg), max_objects=B)
    assert op.size == (b.op.n_observations, b.cfg.setup.n_points)
    gamma = configs.make_gamma(b.cfg)
    assert rel_l2(op.forward(dev(gamma)).cpu().numpy(), forward_quick_cpu(b.op, gamma)) <= TOL
    y = rand_obs(b, B, 9)
    assert rel_l2(op.adjoint(dev(y)).cpu().numpy(), adjoint_quick_cpu(b.op, y)) <= TOL


def test_setup_form_hankel_small_arguments():
    """Points close to the array (|k r| < 16) use the power-series branch of H0^(2)."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from oracle import Absorption, Setup
    from tests.helpers import setup_kwargs
    s = Setup(n_points_axis=(24, 8), delta_axis=(1e-4, 1e-4), z_start=1e-4, n_elements_axis=(6,),
              pitch_axis=(2e-4,), width_axis=(1.8e-4,), n_face_axis=(3,),
              absorption=Absorption("time_causal", 1500.0, 0.0, 0.5, 1.0, 4e6, True))
    cfg = configs.BornConfig("near-field", s, np.linspace(1e6, 4e6, 5), [configs.Wave("qpw", (10.0,))],
                             density=0.2, seed=3)
    b = configs.build(cfg, direct_elements=True)
    op = OperatorBorn.from_setup(**setup_kwargs(cfg), max_objects=1)
    gamma = configs.make_gamma(cfg)
    assert rel_l2(op.forward(dev(gamma)).cpu().numpy(), forward_quick_cpu(b.op, gamma)) <= TOL


def test_plain_c_harness():
    """The C-only driver (no Python in the loop) passes its own dot-product and VJP checks."""
    import json
    import subprocess
    from comp_ui_toolbox_gb300 import build
    exe = build.build_harness()
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert res["ok"] and res["dot_product_rel_err"] < 1e-6


@pytest.mark.parametrize("name", ["c0", "c1", "c2", "ragged"])
def test_bf16x3_tensor_core_matches_oracle(name):
    """Split-BF16 tcgen05 forward and adjoint: relative L2 <= 1e-5 against the FP64 oracle."""
    b = built(name)
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    op.set_precision("bf16x3")
    gamma = configs.make_gamma(b.cfg, complex_values=True)
    u = op.forward(dev(gamma)).cpu().numpy()
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= TOL
    y = rand_obs(b, B, 7)
    g = op.adjoint(dev(y)).cpu().numpy()
    assert rel_l2(g, adjoint_quick_cpu(b.op, y)) <= TOL
    assert op.device_status() == 0


def test_bf16x3_vjp_matches_oracle():
    b = built("c1")
    op = make_operator(b, "lateral", max_objects=1)
    op.set_precision("bf16x3")
    gamma_true = configs.make_gamma(b.cfg)
    u_meas = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 30.0, seed=5)
    gamma = np.random.default_rng(21).standard_normal(gamma_true.shape)
    r = forward_quick_cpu(b.op, gamma) - u_meas
    grad, loss = op.vjp(dev(gamma), dev(u_meas))
    assert rel_l2(grad.cpu().numpy(), adjoint_quick_cpu(b.op, r)) <= TOL


def test_bf16x3_refused_for_3d():
    from comp_ui_toolbox_gb300 import CuiError
    op = make_operator(built("c3"), "lateral", max_objects=1)
    with pytest.raises(CuiError) as ei:
        op.set_precision("bf16x3")
    assert ei.value.status == 2


@pytest.mark.parametrize("wname,n_freq,n_obj", [("2d-gradient", 12, 1), ("2d-batched", 3, 8), ("2d-plain", 8, 5)])
def test_bf16x3_full_lines_match_fp32(wname, n_freq, n_obj):
    """Split-BF16 tensor-core forward and adjoint on full-width benchmark grid lines
    (512 or 256 points, 128 elements; several lines per block, several frequencies
    per block) against the FP32 path of the same plan, which the tests above pin to
    the FP64 oracle within 2e-7.  Bound: relative L2 <= 1e-5."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload(wname)
    w.f = w.f[:n_freq]
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj)
    rng = np.random.default_rng(3)
    g = rng.standard_normal((op.n_points, n_obj)) + 1j * rng.standard_normal((op.n_points, n_obj))
    y = rng.standard_normal((op.n_observations, n_obj)) + 1j * rng.standard_normal((op.n_observations, n_obj))
    u32 = op.forward(dev(g)).cpu().numpy()
    a32 = op.adjoint(dev(y)).cpu().numpy()
    op.set_precision("bf16x3")
    u16 = op.forward(dev(g)).cpu().numpy()
    a16 = op.adjoint(dev(y)).cpu().numpy()
    assert op.device_status() == 0
    assert rel_l2(u16, u32) <= TOL
    assert rel_l2(a16, a32) <= TOL
    # per object, so that a wrong column mapping of one object cannot hide in the total
    for b in range(n_obj):
        assert rel_l2(u16[:, b], u32[:, b]) <= TOL
        assert rel_l2(a16[:, b], a32[:, b]) <= TOL
    op.close()


@pytest.mark.parametrize("name", ["c1", "c3"])
def test_autotune_keeps_a_path_that_matches_oracle(name):
    """cui_born_autotune times the FP32 and (2D) split-BF16 paths, keeps the faster,
    and the plan's outputs stay within the operator's bound."""
    b = built(name)
    op = make_operator(b, "lateral", max_objects=1)
    res = op.autotune(1)
    assert res["ms_fp32"] > 0
    assert (res["ms_bf16x3"] > 0) == (name != "c3")  # the 3D setup has no tensor-core path
    assert res["precision"] in ("fp32", "bf16x3")
    gamma = configs.make_gamma(b.cfg, complex_values=True)
    u = op.forward(dev(gamma)).cpu().numpy()
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= TOL
    assert op.device_status() == 0


@pytest.mark.parametrize("n_lines,n_obj", [(17, 6), (9, 5)])
def test_bf16x3_wide_tiles_partial_tile_and_odd_lines(n_lines, n_obj):
    """64-column tiles (4 objects x 16 waves): the last tile only partly filled (objects not a
    multiple of 4) and an odd number of grid lines (the adjoint's last block covers one line
    of its two).  Compared per object with the FP32 path of the same plan; bound 1e-5."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload("2d-batched")
    w.f = w.f[:2]
    w.n_points_axis = (w.n_points_axis[0], n_lines)
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj)
    rng = np.random.default_rng(5)
    g = rng.standard_normal((op.n_points, n_obj)) + 1j * rng.standard_normal((op.n_points, n_obj))
    y = rng.standard_normal((op.n_observations, n_obj)) + 1j * rng.standard_normal((op.n_observations, n_obj))
    u32 = op.forward(dev(g)).cpu().numpy()
    a32 = op.adjoint(dev(y)).cpu().numpy()
    op.set_precision("bf16x3")
    u16 = op.forward(dev(g)).cpu().numpy()
    a16 = op.adjoint(dev(y)).cpu().numpy()
    assert op.device_status() == 0
    for b in range(n_obj):
        assert rel_l2(u16[:, b], u32[:, b]) <= TOL
        assert rel_l2(a16[:, b], a32[:, b]) <= TOL
    op.close()


@pytest.mark.parametrize("wname,n_lines,n_obj", [("2d-gradient", 9, 1), ("2d-gradient", 17, 1), ("2d-plain", 9, 3)])
def test_bf16x3_narrow_tiles_odd_lines(wname, n_lines, n_obj):
    """16-column tiles, whose adjoint blocks cover two grid lines (two blocks per SM): an odd
    number of lines leaves the last block one line.  11 waves and one object fill 11 of 16
    columns; one wave and three objects give two-object tiles, the last one half empty.
    Compared per object with the FP32 path of the same plan; bound 1e-5."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload(wname)
    w.f = w.f[:3]
    w.n_points_axis = (w.n_points_axis[0], n_lines)
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj)
    rng = np.random.default_rng(7)
    g = rng.standard_normal((op.n_points, n_obj)) + 1j * rng.standard_normal((op.n_points, n_obj))
    y = rng.standard_normal((op.n_observations, n_obj)) + 1j * rng.standard_normal((op.n_observations, n_obj))
    u32 = op.forward(dev(g)).cpu().numpy()
    a32 = op.adjoint(dev(y)).cpu().numpy()
    op.set_precision("bf16x3")
    u16 = op.forward(dev(g)).cpu().numpy()
    a16 = op.adjoint(dev(y)).cpu().numpy()
    assert op.device_status() == 0
    for b in range(n_obj):
        assert rel_l2(u16[:, b], u32[:, b]) <= TOL
        assert rel_l2(a16[:, b], a32[:, b]) <= TOL
    op.close()


def test_bf16x3_launch_shapes_and_autotune():
    """Every launch shape the autotuner can pick for the line-unit kernels (64- or 32-column tiles,
    fewer or more blocks per launch) on a 64-column plan (16 waves, 6 objects, 17 grid lines), and
    the shapes autotune keeps, against the FP32 path of the same plan; bound 1e-5 per object."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload("2d-batched")
    w.f = w.f[:3]
    w.n_points_axis = (w.n_points_axis[0], 17)
    n_obj = 6
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj)
    rng = np.random.default_rng(9)
    g = rng.standard_normal((op.n_points, n_obj)) + 1j * rng.standard_normal((op.n_points, n_obj))
    y = rng.standard_normal((op.n_observations, n_obj)) + 1j * rng.standard_normal((op.n_observations, n_obj))
    u32 = op.forward(dev(g)).cpu().numpy()
    a32 = op.adjoint(dev(y)).cpu().numpy()
    op.set_precision("bf16x3")

    def check():
        u16 = op.forward(dev(g)).cpu().numpy()
        a16 = op.adjoint(dev(y)).cpu().numpy()
        assert op.device_status() == 0
        for b in range(n_obj):
            assert rel_l2(u16[:, b], u32[:, b]) <= TOL
            assert rel_l2(a16[:, b], a32[:, b]) <= TOL

    for shapes in [(0, 0, 0), (1, 0, 0), (0, 4 * 152, 4 * 152), (1, 16 * 152, 16 * 152), (0, 1, 1)]:
        op.set_launch_shapes(*shapes)
        check()
    res = op.autotune(n_obj)
    assert set(res["launch_shapes"]) == {"narrow_tiles", "fwd_blocks", "adj_blocks"}
    if res["precision"] == "bf16x3":
        check()
    op.close()


@pytest.mark.parametrize("name", CONFIGS)
def test_energy_rx_matches_oracle(name):
    """Received energies ||Phi e_p||^2 (energy_rx_canonical, operator_born.m:718-859) against the
    FP64 restatement; bound 1e-5 relative L2."""
    from oracle.born_oracle import energy_rx_cpu
    b = built(name)
    op = make_operator(b, "lateral", max_objects=max(1, b.cfg.n_objects))
    E = op.energy_rx().cpu().numpy()
    assert rel_l2(E, energy_rx_cpu(b.op)) <= TOL
    assert op.device_status() == 0
