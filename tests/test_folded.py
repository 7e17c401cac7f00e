"""GPU parity of the folded-operator path (``bf16x3-folded``): split-BF16 tcgen05 GEMMs against
the observation x grid-point matrix summed over each mix's active elements.

Tolerance: relative L2 <= 1e-5 against the FP64 oracle (``forward_quick_cpu`` /
``adjoint_quick_cpu``, ``operator_born.m:332-596``) on the small configurations, per object,
and against the FP32 path of the same plan on full-width benchmark grid lines (full-length
K ranges, where the accumulation chains matter).
"""

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, configs, forward_quick_cpu
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5
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


@pytest.mark.parametrize("name,B", [("c0", 1), ("c1", 3), ("c2", 8), ("c2", 70), ("ragged", 9), ("c3", 2)])
def test_folded_matches_oracle(name, B):
    """Forward and adjoint per object against the FP64 oracle; 70 objects take two GEMM
    passes, the second one partly filled; the ragged setup has mixes over frequency subsets;
    c3 is a 3D setup with a stored table."""
    b = built(name)
    op = make_operator(b, "lateral", max_objects=B)
    op.set_precision("bf16x3-folded")
    gamma = configs.make_gamma(b.cfg, n_objects=B, seed=31, complex_values=True)
    u_ref = forward_quick_cpu(b.op, gamma)
    y = rand_obs(b, B, 9)
    g_ref = adjoint_quick_cpu(b.op, y)
    u = op.forward(dev(gamma)).cpu().numpy()
    g = op.adjoint(dev(y)).cpu().numpy()
    assert op.device_status() == 0
    for k in range(B):
        assert rel_l2(u[:, k], u_ref[:, k]) <= TOL
        assert rel_l2(g[:, k], g_ref[:, k]) <= TOL
    assert op.refresh_info()["folded_bytes"] > 0
    op.close()


def test_folded_vjp_and_lasso_match_fp32():
    """The VJP and the fused LASSO update on the folded path against the FP32 path."""
    b = built("c2")
    B = 4
    op = make_operator(b, "lateral", max_objects=B)
    gamma_true = configs.make_gamma(b.cfg, n_objects=B, seed=3)
    u_meas = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 30.0, seed=5)
    gamma = np.random.default_rng(21).standard_normal(gamma_true.shape)
    r = forward_quick_cpu(b.op, gamma) - u_meas
    op.set_precision("bf16x3-folded")
    grad, _ = op.vjp(dev(gamma), dev(u_meas))
    assert rel_l2(grad.cpu().numpy(), adjoint_quick_cpu(b.op, r)) <= TOL
    # threshold at 5 % of |Phi^H u|_inf per column (the bench's choice), so that the iterates are not all zero
    lam = torch.from_numpy((0.05 * np.abs(adjoint_quick_cpu(b.op, u_meas)).max(axis=0)).astype(np.float32)).cuda()
    step = 0.5 / op.norm_estimate(8)
    outs = {}
    for prec in ("fp32", "bf16x3-folded"):
        op.set_precision(prec)
        g0 = torch.zeros((B, op.n_points), dtype=torch.complex64, device="cuda")
        u_cols = dev(u_meas).t().contiguous()
        op.lasso_(g0, u_cols, lam, step, 5)
        outs[prec] = g0.cpu().numpy()
    assert np.abs(outs["fp32"]).max() > 0
    assert rel_l2(outs["bf16x3-folded"], outs["fp32"]) <= 1e-4
    assert op.device_status() == 0
    op.close()


@pytest.mark.parametrize("n_freq,n_obj", [(2, 64), (1, 5)])
def test_folded_full_lines_match_fp32(n_freq, n_obj):
    """Full 512 x 512 grid of the batched workload (16 random-apodization waves mixed into 32
    receive signals, 128 elements) at a few frequencies, against the FP32 path of the same
    plan per object: K ranges of all 262144 points (forward) and all rows (adjoint)."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload("2d-batched")
    w.f = w.f[:n_freq]
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=n_obj)
    rng = np.random.default_rng(3)
    g = rng.standard_normal((op.n_points, n_obj)) + 1j * rng.standard_normal((op.n_points, n_obj))
    y = rng.standard_normal((op.n_observations, n_obj)) + 1j * rng.standard_normal((op.n_observations, n_obj))
    u32 = op.forward(dev(g)).cpu().numpy()
    a32 = op.adjoint(dev(y)).cpu().numpy()
    op.set_precision("bf16x3-folded")
    u16 = op.forward(dev(g)).cpu().numpy()
    a16 = op.adjoint(dev(y)).cpu().numpy()
    assert op.device_status() == 0
    for k in range(n_obj):
        assert rel_l2(u16[:, k], u32[:, k]) <= TOL
        assert rel_l2(a16[:, k], a32[:, k]) <= TOL
    op.close()


def test_folded_refused_without_stored_table():
    """Streamed and generated 3D tables cannot be folded (the build reads the stored table)."""
    from comp_ui_toolbox_gb300 import CuiError, OperatorBorn
    from tests.helpers import setup_kwargs

    b = built("c3")
    op = OperatorBorn.from_setup(**setup_kwargs(b.cfg), device=0, max_objects=1, table_storage="streamed")
    with pytest.raises(CuiError) as ei:
        op.set_precision("bf16x3-folded")
    assert ei.value.status == 2
    op.close()


def test_folded_host_vjp_writes_the_callers_array():
    """On a full 512 x 512 grid each adjoint block covers all rows (one K chunk), so in the direct
    host path the GEMM writes the FP64 gradient into the caller's array itself.  It equals the
    device VJP's gradient exactly (the same FP32 values, converted to FP64), for an aligned output
    and for one 8 bytes off a 16-byte boundary, which takes the separate write-back instead."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload

    w = workload("2d-batched")
    w.f = w.f[:2]
    B = 8
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=B)
    op.set_precision("bf16x3-folded")
    rng = np.random.default_rng(12)
    g = np.asfortranarray((rng.standard_normal((op.n_points, B)) + 1j * rng.standard_normal((op.n_points, B))).astype(np.complex64).astype(np.complex128))
    u = np.asfortranarray((rng.standard_normal((op.n_observations, B)) + 1j * rng.standard_normal((op.n_observations, B))).astype(np.complex64).astype(np.complex128))
    grad_d, loss_d = op.vjp(dev(g), dev(u))
    grad_d = grad_d.cpu().numpy().astype(np.complex128)
    grad_h, loss_h = op.vjp(g, u)
    assert np.array_equal(grad_h, grad_d)
    np.testing.assert_allclose(loss_h, loss_d.cpu().numpy(), rtol=1e-6)
    nbytes = g.size * 16
    raw = np.zeros(nbytes + 32, dtype=np.uint8)
    off = (8 - raw.ctypes.data % 16) % 16
    out = raw[off:off + nbytes].view(np.complex128).reshape(g.shape, order="F")
    op.vjp(g, u, out=out)
    assert np.array_equal(out, grad_d)
    assert op.device_status() == 0
    op.close()
