"""Bounded device waits that run out (GPU; no fault, no hang).

Every wait of the tensor-core kernels for an operand stage or an accumulator has a wall-clock
limit (``cui_born_set_wait_limit``).  With a limit of 1 ns, on a plan whose blocks wait for many
operand stages and accumulation chains, some wait runs out: the block drains its copies and
MMAs under their own fixed 1 s limit, frees its tensor memory and raises the plan's status word.  The test checks,
for the line-unit and the folded-operator kernels, that

* ``cui_born_plan_status`` reports CUI_ERR_TIMEOUT (the Python mirror raises CuiError 5);
* a later apply while the status is set leaves the status set (its blocks skip their work);
* reading the status clears it, and with the default limit restored the plan's outputs match
  the FP32 path again (relative L2 <= 1e-5).
"""

import numpy as np
import pytest

from oracle import configs
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x3-folded"])
def test_wait_that_runs_out_raises_the_status_and_the_plan_recovers(precision):
    """A full-width grid (the batched workload at two frequencies, 16 objects), whose blocks wait
    for many stages and chains, with a 1 ns limit: a wait that is not satisfied at once runs out."""
    from comp_ui_toolbox_gb300 import CuiError, OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload
    w = workload("2d-batched")
    w.f = w.f[:2]
    B = 16
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=B)
    g = torch.from_numpy(w.gamma(n_objects=B).astype(np.complex64)).cuda()
    u32 = op.forward(g).cpu().numpy()
    op.set_precision(precision)
    assert rel_l2(op.forward(g).cpu().numpy(), u32) <= 1e-5
    assert op.device_status() == 0
    op.set_wait_limit(1)  # 1 ns
    op.forward(g)
    torch.cuda.synchronize()
    op.set_wait_limit(0)
    op.forward(g)  # the status is still set: the contraction blocks skip their work
    torch.cuda.synchronize()
    with pytest.raises(CuiError) as ei:
        op.device_status()
    assert ei.value.status == 5
    assert op.device_status() == 0  # reading cleared it
    assert rel_l2(op.forward(g).cpu().numpy(), u32) <= 1e-5
    assert op.device_status() == 0
    op.close()


def test_wait_limit_bounds_are_checked_on_the_host():
    from comp_ui_toolbox_gb300 import CuiError
    op = make_operator(configs.build(configs.small_config("c1")), "lateral")
    for bad in (-1, 61 * 10**9):
        with pytest.raises(CuiError) as ei:
            op.set_wait_limit(bad)
        assert ei.value.status == 1
    op.close()
