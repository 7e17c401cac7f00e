"""Device LASSO iterations on problems of the uneven batch against the FP64 ISTA oracle (GPU).

The uneven-batch workload runs 50 proximal-gradient iterations per problem
(``gamma <- S(gamma - t Phi^H (Phi gamma - u), t lambda)``, the plainest member of the
solver family behind ``operator.lq_minimization``, ``+scattering/operator.m:601-790``).
For the two problems of the 256 with the least work (problem 230: 128 x 128 grid, 3 waves,
32 frequencies, 64 elements; problem 127: 128 x 128, 1 wave, 90 frequencies, 64 elements)
the device solution of ``cui_born_lasso`` after 50 iterations, on both precisions, is
compared with ``oracle.solvers.lasso_ista`` on the same data.  The oracle operator is split
over frequencies across spawn workers (``oracle.lasso_split``).

The data: u = Phi gamma_true + complex Gaussian noise at 25 dB SNR (FP64, host), gamma_true
the problem's seeded 2 %-sparse real scatterers; lambda = 0.05 ||Phi^H u||_inf; step
0.9 / ||Phi||^2 with the norm estimated on the device (8 power iterations).  Tolerance:
relative L2 <= 1e-4 between the device and oracle solutions.  That is 50 iterations of the
FP32 (or split-BF16) operator, whose single applies agree with the oracle to about 1e-6.
"""

import numpy as np
import pytest

from tests.helpers import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PROBLEMS = (230, 127)
N_ITER = 50
TOL = 1e-4
_DATA = {}


def problem_data(i):
    """(workload, u, lambda, oracle solution, oracle loss) of problem i, from the FP64 oracle."""
    if i in _DATA:
        return _DATA[i]
    from comp_ui_toolbox_gb300.workloads import lasso_problem
    from oracle.lasso_split import FrequencySplitOracle, lasso_problem_config
    w = lasso_problem(i)
    cfg = lasso_problem_config(w.n_points_axis[0], w.n_elements, w.f, [a[0] for _, a in w.waves], w.density,
                               w.seed, w.name)
    with FrequencySplitOracle(cfg) as orc:
        u0 = orc.forward(w.gamma(n_objects=1).real.astype(np.float64) + 0j)
        rng = np.random.default_rng(1000 + i)
        noise = rng.standard_normal(u0.shape) + 1j * rng.standard_normal(u0.shape)
        u = u0 + noise * (np.linalg.norm(u0) / np.linalg.norm(noise)) * 10 ** (-25 / 20)
        lam = 0.05 * float(np.abs(orc.adjoint(u)).max())
        _DATA[i] = dict(w=w, u=u, lam=lam, orc_cfg=cfg)
    return _DATA[i]


def oracle_solution(i, step):
    d = problem_data(i)
    key = ("sol", step)
    if key not in d:
        from oracle.lasso_split import FrequencySplitOracle
        with FrequencySplitOracle(d["orc_cfg"]) as orc:
            d[key] = orc.lasso(d["u"], d["lam"], step, N_ITER)
    return d[key]


@pytest.mark.parametrize("i", PROBLEMS)
def test_lasso_batch_problem_matches_ista(i):
    from comp_ui_toolbox_gb300 import OperatorBorn
    d = problem_data(i)
    w = d["w"]
    op = OperatorBorn.from_setup(**w.setup_kwargs(), device=0, max_objects=1)
    step = 0.9 / op.norm_estimate(8)
    g_ref, loss_ref = oracle_solution(i, step)
    assert np.abs(g_ref).max() > 0  # the threshold leaves scatterers standing
    u = torch.from_numpy(d["u"].astype(np.complex64)).cuda()
    for precision in ("fp32", "bf16x3"):
        op.set_precision(precision)
        g, _ = op.lasso(u, d["lam"], step, N_ITER)
        g = g.cpu().numpy().reshape(-1)
        assert rel_l2(g, g_ref[:, 0]) <= TOL, precision
        assert op.device_status() == 0
    op.close()
