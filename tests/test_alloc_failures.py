"""Cleanup paths under device-allocation failures (GPU: plan creation allocates device memory).

``CUI_BORN_FAIL_ALLOC=N`` makes the N-th device allocation of each plan fail as an out-of-memory
error would (before cudaMalloc is called).  For every N up to the plan's allocation count, plan
creation must return CUI_ERR_OOM and leave the device's free memory where it was; a precision
switch that fails the same way must leave the plan working on its previous path.
"""

import numpy as np
import pytest

from oracle import adjoint_quick_cpu, configs, forward_quick_cpu
from tests.helpers import make_operator, rel_l2, setup_kwargs

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SLACK = 4 << 20  # bytes of free-memory drift tolerated (driver bookkeeping)


def _free():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("form", ["table", "setup"])
def test_every_failed_allocation_of_plan_creation_is_clean(form, monkeypatch):
    from comp_ui_toolbox_gb300 import CuiError, OperatorBorn
    b = configs.build(configs.small_config("c2"))
    create = (lambda: make_operator(b, "lateral", max_objects=b.cfg.n_objects)) if form == "table" else \
        (lambda: OperatorBorn.from_setup(**setup_kwargs(b.cfg), device=0, max_objects=b.cfg.n_objects))
    gamma = configs.make_gamma(b.cfg)
    g = torch.from_numpy(gamma.astype(np.complex64)).cuda()
    op = create()  # warm: first-use loads of kernel modules (the library's and torch's) are outside the measurement
    op.forward(g).cpu()
    op.close()
    free0 = _free()
    n = 1
    while n < 200:
        monkeypatch.setenv("CUI_BORN_FAIL_ALLOC", str(n))
        try:
            op = create()
        except CuiError as e:
            assert e.status == 3, e
            assert "injected allocation failure" in str(e)
            assert abs(_free() - free0) <= SLACK, n
            n += 1
            continue
        break
    monkeypatch.delenv("CUI_BORN_FAIL_ALLOC")
    assert n > 5  # several allocations were failed one at a time
    u = op.forward(g).cpu().numpy()
    assert rel_l2(u, forward_quick_cpu(b.op, gamma)) <= 1e-5
    op.close()
    assert abs(_free() - free0) <= SLACK


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x3-folded"])
def test_failed_precision_switch_keeps_the_plan_working(precision, monkeypatch):
    """Fail the j-th allocation of the switch for j = 1, 2, ... until it succeeds."""
    from comp_ui_toolbox_gb300 import CuiError
    b = configs.build(configs.small_config("c2"))
    op = make_operator(b, "lateral", max_objects=b.cfg.n_objects)
    gamma = configs.make_gamma(b.cfg)
    g = torch.from_numpy(gamma.astype(np.complex64)).cuda()
    u_ref = forward_quick_cpu(b.op, gamma)
    failures = 0
    for j in range(1, 100):
        n0 = op.refresh_info()["device_allocations"]
        monkeypatch.setenv("CUI_BORN_FAIL_ALLOC", str(n0 + j))
        try:
            op.set_precision(precision)
        except CuiError as e:
            assert e.status == 3
            failures += 1
            monkeypatch.delenv("CUI_BORN_FAIL_ALLOC")
            assert rel_l2(op.forward(g).cpu().numpy(), u_ref) <= 1e-5  # still the previous path
            continue
        break
    monkeypatch.delenv("CUI_BORN_FAIL_ALLOC", raising=False)
    assert failures >= 1
    assert op.precision == precision  # a later switch built what the failed ones could not
    assert rel_l2(op.forward(g).cpu().numpy(), u_ref) <= 1e-5
    assert op.device_status() == 0
    op.close()


def test_failed_staging_allocation_then_host_vjp_succeeds(monkeypatch):
    """The FP64 host entry points allocate their device staging buffers on first use.  Fail the
    j-th of those allocations for j = 1, 2, ...: each failed call returns CUI_ERR_OOM, and the next
    call on the same plan allocates only the buffers still missing.  The gradient of the call that
    succeeds is the oracle's (bound 1e-5)."""
    from comp_ui_toolbox_gb300 import CuiError
    b = configs.build(configs.small_config("c1"))
    op = make_operator(b, "lateral", max_objects=1)
    gamma_true = configs.make_gamma(b.cfg)
    u_meas = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 30.0, seed=5)
    gamma = np.random.default_rng(21).standard_normal(gamma_true.shape) + 0j
    grad_ref = adjoint_quick_cpu(b.op, forward_quick_cpu(b.op, gamma) - u_meas)
    failures = 0
    for j in range(1, 20):
        n0 = op.refresh_info()["device_allocations"]
        monkeypatch.setenv("CUI_BORN_FAIL_ALLOC", str(n0 + j))
        try:
            grad, _ = op.vjp(gamma, u_meas)
        except CuiError as e:
            assert e.status == 3, e
            assert "injected allocation failure" in str(e)
            failures += 1
            continue
        finally:
            monkeypatch.delenv("CUI_BORN_FAIL_ALLOC")
        break
    assert failures >= 1
    assert rel_l2(np.asarray(grad), grad_ref) <= 1e-5
    grad, _ = op.vjp(gamma, u_meas)  # the buffers are kept: no further allocation
    assert rel_l2(np.asarray(grad), grad_ref) <= 1e-5
    assert op.device_status() == 0
    op.close()
