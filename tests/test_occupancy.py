"""Occupancy compaction of the FP32 forward (GPU).

The reference's forward contracts only the grid points where some column of gamma is nonzero
(``operator_born.m:361``, ``combined_quick_gpu.cu:457-499``).  The library lists those points on
the device and, when at most the plan's limit (default N_points / 16 with a stored table, / 32 with
a streamed or generated one) are occupied, contracts over the list instead of the dense grid, the
occupied points split into chunks whose partial sums are added in a fixed order.  Checks against the FP64 oracle (relative L2 <= 1e-5 per
column) and against the dense kernels of the same plan: sparse and ragged occupancy, several
columns whose union decides, an all-zero gamma, a union above the limit (the dense path runs),
3D plans with stored, streamed and generated tables, and the LASSO loop whose iterates the
soft threshold makes sparse.
"""

import numpy as np
import pytest

from oracle import configs, forward_quick_cpu
from tests.helpers import make_operator, rel_l2, setup_kwargs

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5


def dev(x):
    return torch.from_numpy(np.asarray(x, dtype=np.complex64)).cuda()


def sparse_gamma(P, B, n_occ, seed):
    rng = np.random.default_rng(seed)
    g = np.zeros((P, B), dtype=np.complex128)
    for b in range(B):
        idx = rng.choice(P, n_occ, replace=False)
        g[idx, b] = rng.standard_normal(n_occ) + 1j * rng.standard_normal(n_occ)
    return g


@pytest.mark.parametrize("name,B", [("c0", 1), ("c1", 1), ("c2", 3), ("ragged", 2), ("c3", 1)])
def test_compacted_forward_matches_oracle_and_dense(name, B):
    b = configs.build(configs.small_config(name))
    op = make_operator(b, "lateral", max_objects=B)
    P = b.op.setup.n_points
    g = sparse_gamma(P, B, max(1, P // (16 * B) - 1), seed=5)  # union below the default limit
    u_ref = forward_quick_cpu(b.op, g)
    u_sparse = op.forward(dev(g)).cpu().numpy()
    op.set_occupancy_limit(0)
    u_dense = op.forward(dev(g)).cpu().numpy()
    for k in range(B):
        assert rel_l2(u_sparse[:, k], u_ref[:, k]) <= TOL
        assert rel_l2(u_sparse[:, k], u_dense[:, k]) <= TOL
    op.set_occupancy_limit(P)  # always compacted, also for a dense gamma
    gd = sparse_gamma(P, B, P // 2, seed=6)
    ud = op.forward(dev(gd)).cpu().numpy()
    assert rel_l2(ud, forward_quick_cpu(b.op, gd)) <= TOL
    op.close()


def test_zero_gamma_and_union_above_the_limit():
    b = configs.build(configs.small_config("c1"))
    op = make_operator(b, "lateral", max_objects=2)
    P = b.op.setup.n_points
    assert not np.any(op.forward(dev(np.zeros((P, 2)))).cpu().numpy())
    # each column sparse, their union above P / 16: the dense kernels run
    g = sparse_gamma(P, 2, P // 20, seed=7)
    assert rel_l2(op.forward(dev(g)).cpu().numpy(), forward_quick_cpu(b.op, g)) <= TOL
    op.close()


@pytest.mark.parametrize("storage", ["stored", "streamed", "generated"])
def test_compacted_forward_on_3d_table_storages(storage):
    from comp_ui_toolbox_gb300 import OperatorBorn
    b = configs.build(configs.small_config("c3"))
    op = OperatorBorn.from_setup(**setup_kwargs(b.cfg), device=0, max_objects=1, table_storage=storage)
    P = b.op.setup.n_points
    g = sparse_gamma(P, 1, P // 32, seed=8)
    assert rel_l2(op.forward(dev(g)).cpu().numpy(), forward_quick_cpu(b.op, g)) <= TOL
    op.close()


def test_lasso_with_compacted_forwards_matches_dense():
    b = configs.build(configs.small_config("c1"))
    gamma_true = configs.make_gamma(b.cfg)
    u = configs.add_noise(forward_quick_cpu(b.op, gamma_true), 25.0, seed=3)
    out = {}
    for limit in (-1, 0):
        op = make_operator(b, "lateral", max_objects=1)
        op.set_occupancy_limit(limit)
        step = 0.9 / op.norm_estimate(8)
        lam = 0.2 * float(np.abs(op.adjoint(dev(u)).cpu().numpy()).max())
        g, _ = op.lasso(dev(u), lam, step, 30)
        out[limit] = g.cpu().numpy()
        op.close()
    assert np.abs(out[0]).max() > 0
    assert rel_l2(out[-1], out[0]) <= 1e-4


@pytest.mark.parametrize("name,storage", [("2d-gradient", "auto"), ("3d", "streamed")])
def test_compacted_forward_at_the_limit_full_size(name, storage):
    """Full-size plans with exactly the default limit's number of occupied points (the longest
    sums the compacted forward forms) against the dense kernels of the same plan (which the
    full-size parity tests pin to the FP64 oracle)."""
    from comp_ui_toolbox_gb300 import OperatorBorn
    from comp_ui_toolbox_gb300.workloads import workload
    w = workload(name)
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=1, table_storage=storage)
    P = op.n_points
    n_occ = P // (16 if op.table_storage == "stored" else 32)
    g = dev(sparse_gamma(P, 1, n_occ, 41))
    u = op.forward(g).cpu().numpy()
    op.set_occupancy_limit(0)
    u_dense = op.forward(g).cpu().numpy()
    assert rel_l2(u, u_dense) <= TOL
    op.set_occupancy_limit(n_occ - 1)  # one point above the limit: the dense kernels run
    assert rel_l2(op.forward(g).cpu().numpy(), u_dense) == 0.0
    op.close()
