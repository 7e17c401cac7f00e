"""The forward entry point that allocates nothing (cui_born_forward_static).

Some callers cannot call cudaMalloc when they apply the operator: plug-in hosts that give a
plug-in a fixed device-memory budget and refuse any further allocation, and real-time loops that
must not enter the allocator (which may synchronise the device) between frames.  This entry point
serves them: its partial sums live in a fixed device array inside the library, and it always
runs the FP32 CUDA-core kernels.  Its results are compared with the existing entry point
(cui_born_forward) and with the FP64 oracle (forward_quick_cpu), on two calls in a row, within the
1e-5 relative L2 tolerance of every parity test here.  This file is collected last so that a
failure here cannot hide an earlier one; it also passes on its own in a fresh process.
"""

import numpy as np
import pytest

from oracle import Setup, configs, forward_quick_cpu
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # the tolerance every parity test of this library uses


def _static_forward(op, g):
    """Call cui_born_forward_static through the C-ABI; g is (P, B) complex64 on the GPU."""
    gc = g.t().contiguous()
    B, P = gc.shape
    out = torch.empty((B, op.n_observations), dtype=torch.complex64, device="cuda")
    st = op._lib.cui_born_forward_static(op._plan, gc.data_ptr(), P, B, out.data_ptr(), op.n_observations,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == 0, op._lib.cui_last_error()
    return out.t()


@pytest.mark.parametrize("name,precision", [("c1", "fp32"), ("c2", "fp32"), ("c2", "bf16x3"), ("c3", "fp32")])
def test_static_forward_matches_forward_and_oracle_twice(name, precision):
    """2D and 3D stored tables; on a plan switched to split-BF16 the static entry still runs FP32."""
    b = configs.build(configs.small_config(name))
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    op.set_precision(precision)
    for seed in (1, 2):  # two calls in a row: the shared array keeps the last call's contents
        gamma = configs.make_gamma(b.cfg, seed=seed)
        g = torch.from_numpy(gamma.astype(np.complex64)).cuda()
        u_fwd = op.forward(g)
        u = _static_forward(op, g)
        torch.cuda.synchronize()
        assert rel_l2(u.cpu().numpy(), u_fwd.cpu().numpy()) <= TOL
        assert rel_l2(u.cpu().numpy(), forward_quick_cpu(b.op, gamma)) <= TOL
    op.close()


def test_static_forward_rejects_sizes_beyond_the_array():
    b = configs.build(configs.small_config("c2"))
    op = make_operator(b, "lateral", max_objects=b.cfg.n_objects)
    P = b.cfg.setup.n_points
    # slots x objects x elements x 16 B above 16 MiB: 32 slots x 16 elements x 16 B = 8 KiB per object
    n_obj = (16 << 20) // (op.info["n_slots"] * op.info["n_elements"] * 16) + 1
    g = torch.zeros((n_obj, P), dtype=torch.complex64, device="cuda")
    out = torch.empty((n_obj, op.n_observations), dtype=torch.complex64, device="cuda")
    st = op._lib.cui_born_forward_static(op._plan, g.data_ptr(), P, n_obj, out.data_ptr(), op.n_observations,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == 1
    assert b"16 MiB" in op._lib.cui_last_error()
    op.close()


def test_static_forward_rejects_more_objects_than_one_launch_covers():
    """A plan so small that 65536 objects fit the array: the launch's z extent (65535) is the limit."""
    s = Setup(n_points_axis=(20, 6), delta_axis=(1e-4, 1e-4), z_start=2e-3, n_elements_axis=(4,),
              pitch_axis=(2e-4,), width_axis=(1.8e-4,), n_face_axis=(1,))
    cfg = configs.BornConfig("tiny-1w", s, np.linspace(3e6, 5e6, 2), [configs.Wave("qpw", (0.0,))], seed=9)
    b = configs.build(cfg)
    op = make_operator(b, "lateral", max_objects=1)
    assert op.info["n_slots"] * op.info["n_elements"] * 16 * 65536 <= 16 << 20
    P, n_obj = b.cfg.setup.n_points, 65536
    g = torch.zeros((n_obj, P), dtype=torch.complex64, device="cuda")
    out = torch.empty((n_obj, op.n_observations), dtype=torch.complex64, device="cuda")
    st = op._lib.cui_born_forward_static(op._plan, g.data_ptr(), P, n_obj, out.data_ptr(), op.n_observations,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == 1
    assert b"65535" in op._lib.cui_last_error()
    op.close()
