"""CPU restatement of semi-discrete optimal transport on Laguerre cells.

Test infrastructure only: the product never imports this module.

The reference's solver (exploragram's OptimalTransportMap3d) is not in the
reference checkout; its only trace is the compute_OTM program
src/examples/exploragram/compute_OTM/main.cpp:280-296 (set_points,
set_epsilon, optimize).  This module restates the published method it
implements (B. Levy, "A numerical algorithm for L2 semi-discrete optimal
transport in 3D", ESAIM M2AN 49(6), 2015, bibliography/geogram.bib:697-702;
the damped Newton of Kitagawa, Merigot and Thibert, JEMS 2019) on top of the
oracle's cells, which are pinned to the reference's ConvexCell:

  cells       every seed's Laguerre cell in the unit cube, clipped by ALL
              other seeds (no security radius, so any weight spread is
              exact): orc_cells with k0 = n - 1, check_sr = 0
  gradient    g_i = nu_i - |Lag_i(w)|
  Hessian     d|Lag_i| / d w_j = -A_ij / (2 |p_i - p_j|) (j != i),
              diagonal = minus the row sum (a graph Laplacian)
  Newton      solve H x = nu - vol by Jacobi-preconditioned CG in FP64 to
              a relative residual of 1e-3, halve the step until every cell
              keeps at least eps0 and the residual norm drops by
              (1 - alpha / 2), the first trial being min(1, 4 x the
              previous step)

Parity for optimal transport is unpinned: the reference's solver and its
test data are absent.  What pins it here is structure: the Hessian against
finite differences of the pinned cell volumes, the known answer of a
lattice (w = 0 is optimal), and convergence to the mass tolerance measured
with the pinned volumes.
"""
from __future__ import annotations

import numpy as np

from . import oracle


def laguerre_cells(xyz: np.ndarray, w: np.ndarray, nthreads: int = 4) -> dict:
    """Exact Laguerre cells in the unit cube (every seed clips every cell)."""
    n = len(xyz)
    return oracle.cells(xyz, w, k0=n - 1, check_sr=False, exact=True, nthreads=nthreads,
                        max_nbr=160)


def hessian(xyz: np.ndarray, c: dict):
    """(rowptr, col, val, diag): the Laplacian with c_ij = (A_ij + A_ji) / (4 d_ij),
    val = -c_ij, diag_i = sum_j c_ij; a facet seen from one side only is dropped."""
    rp = c["rowptr"].astype(np.int64)
    col = c["nbr"].astype(np.int64)
    area = c["area"]
    n = len(xyz)
    row = np.repeat(np.arange(n), np.diff(rp))
    key = row * n + col
    tkey = col * n + row
    order = np.argsort(key)
    pos = np.searchsorted(key[order], tkey)
    pos = np.minimum(pos, len(key) - 1)
    has_t = key[order][pos] == tkey
    a_t = np.where(has_t, area[order][pos], 0.0)
    d = np.sqrt(((xyz[row] - xyz[col]) ** 2).sum(1))
    cc = np.where(has_t, (area + a_t) / (4.0 * d), 0.0)
    diag = np.zeros(n)
    np.add.at(diag, row, cc)
    return rp, col, -cc, diag


def spmv(H, x: np.ndarray) -> np.ndarray:
    rp, col, val, diag = H
    n = len(diag)
    row = np.repeat(np.arange(n), np.diff(rp))
    y = diag * x
    np.add.at(y, row, val * x[col])
    return y


def pcg(H, b: np.ndarray, rtol: float, max_iter: int):
    """Jacobi-preconditioned CG on the mean-zero subspace; (x, iterations)."""
    diag = H[3]
    dinv = np.where(diag > 0, 1.0 / np.where(diag > 0, diag, 1.0), 1.0)
    x = np.zeros_like(b)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    it = 0
    for it in range(1, max_iter + 1):
        Ap = spmv(H, p)
        pAp = p @ Ap
        if not pAp > 0:
            break
        a = rz / pAp
        x += a * p
        r -= a * Ap
        if np.linalg.norm(r) <= rtol * bn:
            break
        z = dinv * r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x - x.mean(), it


def separable_start(xyz: np.ndarray, box_min=(0.0, 0.0, 0.0), box_max=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Starting weights from the seeds' marginal distributions (no reference
    counterpart: the reference's solver starts from zero).

    w = |p|^2 - 2 phi(p) with phi(p) = sum_a Phi_a(p_a), where Phi_a' = F_a
    is the piecewise-linear interpolation of the empirical CDF of axis a
    (rank k of n -> (k + 1/2) / n, mapped onto the box's extent).  For
    product measures grad phi is the Brenier map onto the uniform box.

    No cell of distinct seeds is empty.  Seed i's cell is the set of x where
    x.p_i - phi(p_i) is largest over the seeds (the power distance
    |x - p|^2 - w rearranged), and at x = grad phi(p_i) convexity gives
    x.p_j - phi(p_j) < x.p_i - phi(p_i) for every j != i, strictly because
    each Phi_a is strictly convex between distinct coordinates.  That x lies
    strictly inside the box since 0 < F_a < 1, so the cell keeps a
    neighbourhood of it.  Returned with mean zero."""
    x = np.asarray(xyz, np.float64)
    n = len(x)
    w = (x * x).sum(1)
    for a in range(3):
        order = np.argsort(x[:, a], kind="stable")
        s = x[order, a]
        F = box_min[a] + (np.arange(n) + 0.5) / n * (box_max[a] - box_min[a])
        Phi = np.concatenate([[0.0], np.cumsum(np.diff(s) * 0.5 * (F[1:] + F[:-1]))])
        w[order] -= 2.0 * Phi
    return w - w.mean()


def newton(xyz: np.ndarray, nu: np.ndarray | None = None, w0: np.ndarray | None = None,
           tol: float = 1e-6, max_newton: int = 60, max_cg: int = 4000, nthreads: int = 4,
           cg_rtol: float = 1e-3, step_growth: float = 4.0):
    """Damped Newton from w0 (zeros) to max_i |vol_i - nu_i| / nu_i < tol.

    Returns (w, info) with info = dict(iters, converged, mass_error_inf,
    cell_calls)."""
    n = len(xyz)
    nu = np.full(n, 1.0 / n) if nu is None else np.asarray(nu, np.float64)
    w = np.zeros(n) if w0 is None else np.array(w0, np.float64)
    c = laguerre_cells(xyz, w, nthreads)
    calls = 1
    r = c["vol"] - nu
    err = np.max(np.abs(r) / nu)
    eps0 = 0.5 * min(nu.min(), c["vol"].min())
    it = 0
    alpha_prev = 1.0
    while err >= tol and it < max_newton:
        it += 1
        H = hessian(xyz, c)
        b = -(r - r.mean())
        x, _ = pcg(H, b, cg_rtol, max_cg)
        alpha = min(1.0, step_growth * alpha_prev) if step_growth > 0 else 1.0
        for _ in range(30):
            wt = w + alpha * x
            ct = laguerre_cells(xyz, wt, nthreads)
            calls += 1
            rt = ct["vol"] - nu
            if ct["vol"].min() >= eps0 and \
                    np.linalg.norm(rt) <= (1.0 - 0.5 * alpha) * np.linalg.norm(r):
                w, c, r = wt, ct, rt
                alpha_prev = alpha
                break
            alpha *= 0.5
        else:
            break
        err = np.max(np.abs(r) / nu)
    return w, dict(iters=it, converged=bool(err < tol), mass_error_inf=float(err),
                   cell_calls=calls)
