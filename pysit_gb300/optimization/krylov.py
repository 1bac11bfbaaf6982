"""Krylov solvers for the Gauss-Newton system (the reference takes them from pyamg.krylov,
which is not a dependency here).

``gmres`` is restarted GMRES (Saad and Schultz, SIAM J. Sci. Stat. Comput. 7(3), 1986):
Arnoldi with modified Gram-Schmidt, the small least-squares problem solved by Givens
rotations.  It keeps pyamg's calling convention as GaussNewton uses it
(pysit/optimization/gauss_newton.py:62-63): ``gmres(A, b, x0=None, tol=1e-5,
restrt=None, maxiter=None, residuals=None) -> (x, info)``; without ``restrt`` one cycle
of up to ``maxiter`` iterations runs, otherwise ``maxiter`` cycles of ``restrt``; the
stopping test is ||b - A x|| <= tol ||b|| (the rotated least-squares residual inside a
cycle, the explicit one before a restart); info 0 = converged, > 0 = iterations run
without converging, < 0 = breakdown.  ``residuals`` (a list) receives ||r|| after every
iteration, starting with the initial residual.

``cg`` is the conjugate-gradient method (Hestenes and Stiefel, 1952) with the same
convention, for symmetric positive definite operators such as the Gauss-Newton Hessian.
``A`` is anything with ``matvec`` or a callable.
"""
from __future__ import annotations

import numpy as np

__all__ = ["gmres", "cg"]


def _op(A):
    if hasattr(A, "matvec"):
        return A.matvec
    if callable(A):
        return A
    return lambda v: np.asarray(A) @ v


def gmres(A, b, x0=None, tol=1e-5, restrt=None, maxiter=None, residuals=None, callback=None):
    mv = _op(A)
    b = np.asarray(b, dtype=float).reshape(-1)
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=float).reshape(-1)
    if maxiter is None:
        maxiter = min(n, 100)
    if restrt is None:
        cycles, m = 1, int(min(maxiter, n))
    else:
        cycles, m = int(maxiter), int(min(restrt, n))
    normb = np.linalg.norm(b)
    if normb == 0.0:
        normb = 1.0
    r = b - np.asarray(mv(x), dtype=float).reshape(-1)
    beta = np.linalg.norm(r)
    if residuals is not None:
        residuals[:] = [beta]
    if beta <= tol * normb:
        return x, 0
    its = 0
    res = beta
    for cyc in range(cycles):
        V = np.zeros((m + 1, n))
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        V[0] = r / beta
        j_done = 0
        for j in range(m):
            w = np.asarray(mv(V[j]), dtype=float).reshape(-1)
            for i in range(j + 1):  # modified Gram-Schmidt
                H[i, j] = np.dot(V[i], w)
                w = w - H[i, j] * V[i]
            hn = np.linalg.norm(w)
            H[j + 1, j] = hn
            for i in range(j):  # earlier rotations on the new column
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = np.hypot(H[j, j], H[j + 1, j])
            if den == 0.0:
                return x, -1
            cs[j], sn[j] = H[j, j] / den, H[j + 1, j] / den
            H[j, j] = den
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            its += 1
            j_done = j + 1
            res = abs(g[j + 1])
            if residuals is not None:
                residuals.append(res)
            if res <= tol * normb:
                break
            if hn == 0.0:  # the Krylov space is invariant: x is exact in it
                break
            V[j + 1] = w / hn
        y = np.linalg.solve(np.triu(H[:j_done, :j_done]), g[:j_done])
        x = x + V[:j_done].T @ y
        if callback is not None:
            callback(x)
        if cyc == cycles - 1:  # no restart follows: the rotated residual decides (no extra product)
            return x, 0 if res <= tol * normb else its
        r = b - np.asarray(mv(x), dtype=float).reshape(-1)
        beta = np.linalg.norm(r)
        if beta <= tol * normb:
            return x, 0
    return x, its


def cg(A, b, x0=None, tol=1e-5, maxiter=None, residuals=None, callback=None):
    mv = _op(A)
    b = np.asarray(b, dtype=float).reshape(-1)
    n = b.size
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=float).reshape(-1)
    if maxiter is None:
        maxiter = n
    normb = np.linalg.norm(b)
    if normb == 0.0:
        normb = 1.0
    r = b - np.asarray(mv(x), dtype=float).reshape(-1)
    p = r.copy()
    rr = float(np.dot(r, r))
    if residuals is not None:
        residuals[:] = [np.sqrt(rr)]
    if np.sqrt(rr) <= tol * normb:
        return x, 0
    for it in range(1, int(maxiter) + 1):
        Ap = np.asarray(mv(p), dtype=float).reshape(-1)
        pAp = float(np.dot(p, Ap))
        if pAp <= 0.0:
            return x, -1
        a = rr / pAp
        x = x + a * p
        r = r - a * Ap
        rr_new = float(np.dot(r, r))
        if residuals is not None:
            residuals.append(np.sqrt(rr_new))
        if callback is not None:
            callback(x)
        if np.sqrt(rr_new) <= tol * normb:
            return x, 0
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, int(maxiter)
