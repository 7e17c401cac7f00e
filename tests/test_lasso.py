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


def _omp_problem(name, n_scatterers, seed):
    b = configs.build(configs.small_config(name))
    P = b.cfg.setup.n_points
    rng = np.random.default_rng(seed)
    g = np.zeros((P, 1), dtype=np.complex128)
    idx = rng.choice(P, n_scatterers, replace=False)
    g[idx, 0] = (2.0 + np.arange(n_scatterers)) * np.exp(2j * np.pi * rng.random(n_scatterers))
    from oracle import forward_quick_cpu
    return b, forward_quick_cpu(b.op, g)[:, 0], idx, g[idx, 0]


def test_oracle_omp_properties():
    """Residuals fall monotonically, the first atom is a true scatterer, the
    least-squares fit on the true support reproduces the data exactly, and the
    relative-RMSE rule stops the iterations."""
    from oracle.solvers import omp_cpu
    b, y, idx, amp = _omp_problem("c1", 3, 0)
    atoms, coeff, rel = omp_cpu(b.op, y, 5)
    assert len(atoms) == 5 and len(set(atoms.tolist())) == 5
    assert np.all(np.diff(rel) <= 1e-12) and rel[-1] < rel[0] < 1.0
    assert atoms[0] in idx
    _, c_true, rel_true, _ = omp_cpu(b.op, y, 3, path=idx)
    assert rel_true[-1] < 1e-10
    np.testing.assert_allclose(c_true, amp, rtol=1e-8)
    _, _, rel_same, s_same = omp_cpu(b.op, y, 5, path=atoms)
    np.testing.assert_array_equal(rel_same, rel)
    np.testing.assert_array_equal(s_same, np.ones(5))
    a2, _, rel2 = omp_cpu(b.op, y, 5, rel_rmse=rel[1])
    assert len(a2) == 2 and rel2[-1] <= rel[1]


# seeds whose argmax at each of the first 5 steps leads the runner-up by >= 1 %
_OMP_SEEDS = {"c1": 0, "c2": 10}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1", "c2"])
def test_omp_matches_oracle(name):
    """Device OMP (cui_born_omp) against the FP64 restatement of omp.m: the same atoms in the
    same order, coefficients within relative L2 1e-4 and relative residuals within 1e-3
    relative (an FP32 least-squares fit on the device)."""
    torch = pytest.importorskip("torch")
    from oracle.solvers import omp_cpu
    b, y, _, _ = _omp_problem(name, 3, _OMP_SEEDS[name])
    n_atoms = 5
    # stop once the fit is exact: past that point the argmax picks among rounding noise
    atoms_ref, coeff_ref, rel_ref = omp_cpu(b.op, y, n_atoms, rel_rmse=1e-4)
    op = make_operator(b, "lateral", max_objects=max(1, b.cfg.n_objects))
    atoms, coeff, rel = op.omp(torch.from_numpy(y.astype(np.complex64)).cuda(), n_atoms, rel_rmse=1e-4)
    assert list(atoms) == list(atoms_ref)
    assert rel_l2(coeff, coeff_ref) <= 1e-4
    np.testing.assert_allclose(rel, rel_ref, rtol=1e-3, atol=1e-5)
    assert op.device_status() == 0


@pytest.mark.gpu
def test_omp_path_is_an_fp64_argmax_within_tolerance():
    """A problem whose argmax margins go down to 2e-4: each atom the device takes is,
    along its own path, within 1e-4 of the FP64 maximum, and the device's coefficients
    and residuals match the FP64 fit on that path.  Early stop at a relative RMSE."""
    torch = pytest.importorskip("torch")
    from oracle.solvers import omp_cpu
    b, y, _, _ = _omp_problem("c1", 3, 11)
    op = make_operator(b, "lateral", max_objects=1)
    y_d = torch.from_numpy(y.astype(np.complex64)).cuda()
    atoms, coeff, rel = op.omp(y_d, 6)
    _, coeff_ref, rel_ref, scores = omp_cpu(b.op, y, 6, path=atoms)
    assert len(set(atoms.tolist())) == len(atoms) == 6
    assert np.all(scores >= 1.0 - 1e-4)
    assert rel_l2(coeff, coeff_ref) <= 1e-4
    np.testing.assert_allclose(rel, rel_ref, rtol=1e-3, atol=1e-5)
    a2, _, rel2 = op.omp(y_d, 6, rel_rmse=float(rel[2]) * 1.0001)
    assert list(a2) == list(atoms[:3]) and rel2[-1] <= rel[2] * 1.0001
    assert op.device_status() == 0
