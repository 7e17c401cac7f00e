"""Greedy sparse recovery on the device -- orthogonal matching pursuit (cui_born_omp)
and compressive sampling matching pursuit (cui_born_cosamp) -- against the FP64
restatements of omp.m and cosamp.m in the oracle.

CPU tests pin the restatements on problems with a known sparse answer (three
point scatterers); GPU tests run the device solvers through the C-ABI and
compare atoms, coefficients and relative residuals.  The selection steps are
discontinuous, so the problems are seeded where every selection leads its
runner-up by >= 0.5 %, far above the FP32 operator's 1e-6 error; a further
test accepts any atom within 1e-4 of the FP64 maximum on a problem with
near-ties.
"""

import numpy as np
import pytest

from oracle import configs
from tests.helpers import make_operator, rel_l2


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


def test_oracle_cosamp_properties():
    """Three scatterers, s = 4: the support is found in two iterations, the fit is exact,
    and the significant atoms carry the true amplitudes, largest first."""
    from oracle.solvers import cosamp_cpu
    b, y, idx, amp = _omp_problem("c1", 3, 0)
    atoms, coeff, rel = cosamp_cpu(b.op, y, 4, 6, rel_rmse=1e-8)
    assert len(rel) == 2 and rel[-1] < 1e-10 and rel[0] > 1e-3
    big = np.abs(coeff) > 1e-6 * np.abs(coeff).max()
    assert sorted(atoms[big].tolist()) == sorted(idx.tolist())
    assert np.all(np.diff(np.abs(coeff)) <= 0)
    order = {int(a): c for a, c in zip(atoms, coeff)}
    np.testing.assert_allclose([order[int(a)] for a in idx], amp, rtol=1e-8)
    a1, _, rel1 = cosamp_cpu(b.op, y, 4, 1)
    assert len(rel1) == 1 and rel1[0] == rel[0] and len(a1) == 4


@pytest.mark.gpu
@pytest.mark.parametrize("name,seed,s,n_iter", [("c1", 0, 4, 6), ("c2", 1, 4, 6), ("c1", 1, 4, 4)])
def test_cosamp_matches_oracle(name, seed, s, n_iter):
    """Device CoSaMP against the FP64 restatement of cosamp.m: the same number of iterations,
    relative residuals within 1e-3 relative (1e-5 absolute), and the same atoms in the same
    order with coefficients within relative L2 1e-4, over the atoms whose FP64 coefficient is
    above 1e-3 of the largest (once the fit is exact the remaining atoms carry rounding noise).
    ("c1", 1) does not converge: its four iterations keep a support of adjacent grid points."""
    torch = pytest.importorskip("torch")
    from oracle.solvers import cosamp_cpu
    b, y, _, _ = _omp_problem(name, 3, seed)
    atoms_ref, coeff_ref, rel_ref = cosamp_cpu(b.op, y, s, n_iter, rel_rmse=1e-4)
    op = make_operator(b, "lateral", max_objects=1)
    y_d = torch.from_numpy(y.astype(np.complex64)).cuda()
    atoms, coeff, rel = op.cosamp(y_d, s, n_iter, rel_rmse=1e-4)
    assert len(rel) == len(rel_ref)
    np.testing.assert_allclose(rel, rel_ref, rtol=1e-3, atol=1e-5)
    nb = int(np.sum(np.abs(coeff_ref) > 1e-3 * np.abs(coeff_ref).max()))
    assert list(atoms[:nb]) == list(atoms_ref[:nb])
    assert rel_l2(coeff[:nb], coeff_ref[:nb]) <= 1e-4
    assert op.device_status() == 0


@pytest.mark.gpu
def test_cosamp_rejects_bad_sizes():
    torch = pytest.importorskip("torch")
    from comp_ui_toolbox_gb300.born import CuiError
    b, y, _, _ = _omp_problem("c1", 3, 0)
    op = make_operator(b, "lateral", max_objects=1)
    y_d = torch.from_numpy(y.astype(np.complex64)).cuda()
    for s in (0, 513, b.cfg.setup.n_points):
        with pytest.raises(CuiError):
            op.cosamp(y_d, s, 2)
