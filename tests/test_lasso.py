"""Proximal-gradient LASSO iterations (cui_born_lasso) against the FP64 oracle.

CPU tests pin the oracle's solver (soft threshold, objective decrease); GPU
tests run the library's device iterations through the C-ABI and compare them
with the oracle, across precisions, and under CUDA-graph capture of several
plans.  Tolerance: relative L2 <= 1e-5 (the operator's bound) after the
iterations, since the soft threshold is 1-Lipschitz and does not amplify the
operator's error.
"""

import numpy as np
import pytest

from oracle import configs
from oracle.solvers import lasso_ista, operator_norm2, soft_threshold
from tests.helpers import make_operator, rel_l2

TOL = 1e-5
N_ITER = 8


def _problem(name, seed=0):
    b = configs.build(configs.small_config(name))
    g_true = configs.make_gamma(b.cfg, seed=seed)
    from oracle import forward_quick_cpu
    u = configs.add_noise(forward_quick_cpu(b.op, g_true), 25.0, seed=seed + 1)
    L = operator_norm2(b.op)
    from oracle import adjoint_quick_cpu
    lam = 0.05 * np.max(np.abs(adjoint_quick_cpu(b.op, u)), axis=0)
    return b, u, lam, 0.9 / L


def test_soft_threshold():
    v = np.array([3 + 4j, 0.1 + 0j, -2j, 0j])
    out = soft_threshold(v, 1.0)
    np.testing.assert_allclose(out, [(3 + 4j) * 0.8, 0, -1j, 0])


def test_oracle_ista_decreases_objective():
    b, u, lam, step = _problem("c1")
    from oracle import forward_quick_cpu

    def objective(g):
        r = forward_quick_cpu(b.op, g) - u
        return 0.5 * np.sum(np.abs(r) ** 2) + lam[0] * np.sum(np.abs(g))

    g1, _ = lasso_ista(b.op, u, lam, step, 2)
    g2, _ = lasso_ista(b.op, u, lam, step, 6)
    assert objective(g2) < objective(g1) < objective(np.zeros_like(g1))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "c2", "ragged"])
def test_lasso_matches_oracle(name):
    torch = pytest.importorskip("torch")
    b, u, lam, step = _problem(name)
    B = u.shape[1]
    op = make_operator(b, "lateral", max_objects=B)
    g_ref, loss_ref = lasso_ista(b.op, u, lam, step, N_ITER)
    g, loss = op.lasso(torch.from_numpy(u.astype(np.complex64)).cuda(), torch.from_numpy(lam.astype(np.float32)),
                       step, N_ITER)
    torch.cuda.synchronize()
    assert rel_l2(g.cpu().numpy(), g_ref) <= TOL
    np.testing.assert_allclose(loss.cpu().numpy(), loss_ref, rtol=1e-4)
    assert op.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "c2"])
def test_lasso_bf16x3_matches_oracle(name):
    torch = pytest.importorskip("torch")
    b, u, lam, step = _problem(name)
    B = u.shape[1]
    op = make_operator(b, "lateral", max_objects=B)
    op.set_precision("bf16x3")
    g_ref, _ = lasso_ista(b.op, u, lam, step, N_ITER)
    g, _ = op.lasso(torch.from_numpy(u.astype(np.complex64)).cuda(), torch.from_numpy(lam.astype(np.float32)),
                    step, N_ITER)
    assert rel_l2(g.cpu().numpy(), g_ref) <= TOL
    assert op.device_status() == 0


@pytest.mark.gpu
def test_lasso_iterations_of_several_plans_in_one_cuda_graph():
    """The iterations allocate nothing and launch only on the given stream: two
    plans captured into one CUDA graph replay to the same result as direct calls."""
    torch = pytest.importorskip("torch")
    probs = [_problem("c1", seed=0), _problem("ragged", seed=3)]
    ops, us, lams, g_direct, g_graph = [], [], [], [], []
    for b, u, lam, step in probs:
        op = make_operator(b, "lateral", max_objects=u.shape[1])
        ops.append(op)
        us.append(torch.from_numpy(u.T.copy().astype(np.complex64)).cuda())
        lams.append(torch.from_numpy(lam.astype(np.float32)).cuda())
        g_direct.append(torch.zeros((u.shape[1], op.n_points), dtype=torch.complex64, device="cuda"))
        g_graph.append(torch.zeros_like(g_direct[-1]))
    for op, u, lam, g, (_, _, _, step) in zip(ops, us, lams, g_direct, probs):
        op.lasso_(g, u, lam, step, N_ITER)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        for op, u, lam, g, (_, _, _, step) in zip(ops, us, lams, g_graph, probs):
            op.lasso_(g, u, lam, step, N_ITER)
    for g in g_graph:
        g.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for a, c in zip(g_direct, g_graph):
        assert torch.equal(a, c)

