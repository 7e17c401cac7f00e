"""FP64 restatement of the solver loop that drives the Born operator (test infrastructure).

TEST INFRASTRUCTURE ONLY: used by ``tests/`` to check the library's
device LASSO iterations (``cui_born_lasso``) and orthogonal matching pursuit
(``cui_born_omp``); nothing in the product imports it.

The reference solves its sparse-recovery problems through
``operator.lq_minimization`` (``+scattering/operator.m:601-790``), which wraps
the operator as ``op_A(x, mode) = combined_scalar(op, mode, x)`` (``:717``) and
hands it to an algorithm object (``:723-726``): SPGL1 (``+regularization/
+algorithms/+convex/spgl1.m:154``, the external spgl1-1.8 package, not vendored)
or OMP/CoSaMP.  Every such iteration is a forward apply, a residual and an
adjoint apply -- the gradient of 0.5||Phi gamma - u||^2.  The uneven-batch
workload runs the plainest member of that family, proximal-gradient LASSO
(ISTA):

    gamma <- S(gamma - t Phi^H (Phi gamma - u), t lambda),  S(v, s) = v max(0, 1 - s/|v|)

which is what :func:`lasso_ista` restates with the oracle's FP64 operator.
:func:`omp_cpu` restates the greedy member, ``omp.m``.
"""

from __future__ import annotations

import numpy as np

from .born_oracle import OperatorTables, adjoint_quick_cpu, forward_quick_cpu


def soft_threshold(v: np.ndarray, s) -> np.ndarray:
    """Complex soft threshold ``v * max(0, 1 - s/|v|)`` (proximal map of ``s * ||v||_1``)."""
    mag = np.abs(v)
    with np.errstate(divide="ignore", invalid="ignore"):
        scale = np.where(mag > s, 1.0 - s / np.where(mag > 0, mag, 1.0), 0.0)
    return v * scale


def lasso_ista(op: OperatorTables, u: np.ndarray, lam, step: float, n_iter: int, gamma0=None,
               forward=None, adjoint=None, n_points: int | None = None):
    """``n_iter`` ISTA iterations per column of ``u``; returns ``(gamma, loss)`` where ``loss``
    is ``0.5||Phi gamma_k - u||^2`` of the last iteration's input iterate (per column).
    ``forward``/``adjoint`` (callables on FP64 arrays, with ``n_points``) replace the oracle
    operator ``op``, e.g. by one split over processes."""
    if forward is None:
        def forward(x):
            return forward_quick_cpu(op, x)

        def adjoint(y):
            return adjoint_quick_cpu(op, y)
    u = np.asarray(u, dtype=np.complex128)
    u2 = u[:, None] if u.ndim == 1 else u
    B = u2.shape[1]
    P = op.setup.n_points if n_points is None else n_points
    g = np.zeros((P, B), dtype=np.complex128) if gamma0 is None else np.array(gamma0, dtype=np.complex128).reshape(P, B)
    lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (B,))
    loss = np.zeros(B)
    for _ in range(n_iter):
        r = forward(g) - u2
        loss = 0.5 * np.sum(np.abs(r) ** 2, axis=0)
        g = soft_threshold(g - step * adjoint(r), step * lam[None, :])
    return g, loss


def operator_norm2(op: OperatorTables, n_iter: int = 30, seed: int = 0) -> float:
    """||Phi||_2^2 by power iteration on Phi^H Phi (FP64)."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((op.setup.n_points, 1)) + 0j
    x /= np.linalg.norm(x)
    lam = 0.0
    for _ in range(n_iter):
        y = adjoint_quick_cpu(op, forward_quick_cpu(op, x))
        lam = float(np.linalg.norm(y))
        x = y / lam
    return lam


def omp_cpu(op: OperatorTables, y: np.ndarray, n_atoms_max: int, rel_rmse: float = 0.0,
            path=None):
    """Orthogonal matching pursuit, restating ``omp.m:161-200`` with the FP64 operator:
    adjoint of the residual (``:166-171``), atom of largest magnitude (``:174``), the
    atom's column via a forward of a unit vector (``:177-185``), the normal equations on
    the atoms so far (``:190-191``) and the residual (``:196-198``); stops once the
    relative RMSE is reached (``:215``).  Returns ``(atoms, coefficients, rel_residuals)``.

    With ``path`` (a sequence of atoms) the iterations take those atoms instead of the
    argmax and the function returns ``(atoms, coefficients, rel_residuals, scores)``,
    ``scores[i]`` being the magnitude of the taken atom in the adjoint of the residual
    divided by the largest magnitude there (1 for an exact argmax).  It evaluates an
    atom sequence chosen by a lower-precision implementation."""
    y = np.asarray(y, dtype=np.complex128).reshape(-1)
    P = op.setup.n_points
    y_norm = np.linalg.norm(y)
    res = y.copy()
    atoms, cols, rel, scores = [], [], [], []
    coeff = np.zeros(0, dtype=np.complex128)
    n_iter = min(n_atoms_max, len(y)) if path is None else len(path)
    for i in range(n_iter):
        g = np.abs(adjoint_quick_cpu(op, res[:, None])[:, 0])
        k = int(np.argmax(g)) if path is None else int(path[i])
        scores.append(g[k] / g.max())
        atoms.append(k)
        e = np.zeros((P, 1))
        e[k] = 1.0
        cols.append(forward_quick_cpu(op, e)[:, 0])
        A = np.stack(cols, axis=1)
        coeff = np.linalg.solve(A.conj().T @ A, A.conj().T @ y)
        res = y - A @ coeff
        rel.append(np.linalg.norm(res) / y_norm)
        if path is None and rel[-1] <= rel_rmse:
            break
    if path is None:
        return np.array(atoms), coeff, np.array(rel)
    return np.array(atoms), coeff, np.array(rel), np.array(scores)


def cosamp_cpu(op: OperatorTables, y: np.ndarray, sparsity: int, n_iter_max: int, rel_rmse: float = 0.0,
               return_margins: bool = False):
    """Compressive sampling matching pursuit, restating ``cosamp.m:174-272`` with the FP64
    operator: signal proxy ``Phi^H r`` (``:180-185``), the ``2 s`` largest magnitudes in a
    stable descending sort (``:188-189``), union with the current atoms in ascending order
    (``:192-195``), the new atoms' columns via forwards of unit vectors (``:209-228``), the
    least-squares fit ``A \\ y`` on the union (``:244``), pruning to the ``s`` largest
    coefficients in a stable descending sort (``:247-249``), the residual with the pruned
    coefficients, not refitted (``:259-261``), and the relative-RMSE stop (``:270``).

    Returns ``(atoms, coefficients, rel_residuals)``: the final ``s`` atoms in the
    reference's order (descending coefficient magnitude) and their coefficients.  With
    ``return_margins`` a fourth item lists, per iteration, the relative gaps at the two
    selection boundaries (2s-th vs next proxy magnitude, s-th vs next coefficient
    magnitude) that decide the sets."""
    y = np.asarray(y, dtype=np.complex128).reshape(-1)
    P = op.setup.n_points
    y_norm = np.linalg.norm(y)
    res = y.copy()
    atoms = np.zeros(0, dtype=np.int64)
    cols = {}
    rel, margins = [], []
    coeff_kept = np.zeros(0, dtype=np.complex128)
    n_sel = min(2 * sparsity, P)
    for _ in range(min(n_iter_max, len(y))):
        g = np.abs(adjoint_quick_cpu(op, res[:, None])[:, 0])
        order = np.argsort(-g, kind="stable")
        ident = order[:n_sel]
        m_sel = (g[order[n_sel - 1]] / g[order[n_sel]] - 1.0) if n_sel < P else np.inf
        union = np.union1d(atoms, ident).astype(np.int64)
        for k in union:
            if int(k) not in cols:
                e = np.zeros((P, 1))
                e[k] = 1.0
                cols[int(k)] = forward_quick_cpu(op, e)[:, 0]
        A = np.stack([cols[int(k)] for k in union], axis=1)
        coeff = np.linalg.lstsq(A, y, rcond=None)[0]
        mag = np.abs(coeff)
        keep = np.argsort(-mag, kind="stable")
        m_prune = (mag[keep[sparsity - 1]] / mag[keep[sparsity]] - 1.0) if sparsity < len(union) else np.inf
        keep = keep[:sparsity]
        atoms = union[keep]
        coeff_kept = coeff[keep]
        cols = {int(k): cols[int(k)] for k in atoms}
        res = y - np.stack([cols[int(k)] for k in atoms], axis=1) @ coeff_kept
        rel.append(np.linalg.norm(res) / y_norm)
        margins.append((m_sel, m_prune))
        if rel[-1] <= rel_rmse:
            break
    out = (atoms, coeff_kept, np.array(rel))
    return out + (margins,) if return_margins else out
