"""The forward entry point that allocates nothing (cui_born_forward_static).

Callers that cannot call cudaMalloc at apply time -- a stream being captured
into a CUDA graph, plug-in hosts with a fixed device-memory budget, real-time
loops -- use this entry point; its partial sums live in a fixed device array
inside the library.  This file is collected last so that a failure here
cannot hide an earlier one; it also passes on its own in a fresh process.
"""

import numpy as np
import pytest

from oracle import configs
from tests.helpers import make_operator, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # the tolerance every FP32 parity test of this library uses


def _static_forward(op, g):
    """Call cui_born_forward_static through the C-ABI; g is (P, B) complex64 on the GPU."""
    gc = g.t().contiguous()
    B, P = gc.shape
    out = torch.empty((B, op.n_observations), dtype=torch.complex64, device="cuda")
    st = op._lib.cui_born_forward_static(op._plan, gc.data_ptr(), P, B, out.data_ptr(), op.n_observations,
                                         torch.cuda.current_stream().cuda_stream)
    assert st == 0, op._lib.cui_last_error()
    return out.t()


@pytest.mark.parametrize("name", ["c1", "c2"])
def test_static_forward_matches_forward_twice(name):
    b = configs.build(configs.small_config(name))
    B = b.cfg.n_objects
    op = make_operator(b, "lateral", max_objects=B)
    for seed in (1, 2):  # two calls in a row: the shared array keeps the last call's contents
        g = torch.from_numpy(configs.make_gamma(b.cfg, seed=seed).astype(np.complex64)).cuda()
        u_ref = op.forward(g)
        u = _static_forward(op, g)
        torch.cuda.synchronize()
        assert rel_l2(u.cpu().numpy(), u_ref.cpu().numpy()) <= TOL


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
