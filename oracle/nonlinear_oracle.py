"""Oracle of the nonlinear DG operator S(u) = A u + R(u), its Jacobian and
Newton's method.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker; the product never
imports it.

- A u: the oracle's restatement of the GalerkinOperator apply (oracle.cpp).
- R(u)_l = int_K r(u_h) phi_l with r(u) = c1 u + c3 u^3 + ce e^u, by the tensor
  Gauss rule of the oracle (pinned to the reference's GaussPts) and its
  Legendre polynomials (pinned to LegendrePolynomials): the volume integral of
  GalerkinOperator (schemes/galerkin.hh:332-360) for the integrand r(u) v,
  here as a direct (not sum-factorised) evaluation at every point.
- newton(): NewtonInverseOperator::operator() (solver/newtoninverseoperator.hh:
  688-790) with lineSearch (:588-630), failed() (:570-586) and
  EisenstatWalkerStrategy::nextLinearTolerance (:64-81), restated in Python.
"""
import math

import numpy as np

import oracle


class NonlinearProblem:
    """reaction: the coefficients (c1, c3, ce) of the built-in family, or a
    pair of callables (r, dr) of (u, x, y, z) for a user-defined reaction."""

    def __init__(self, prob, reaction):
        self.prob = prob
        self.user = callable(reaction[0])
        if self.user:
            self.ufun, self.udfun = reaction
        else:
            self.c1, self.c3, self.ce = (float(c) for c in reaction)
        n, q = prob.order + 1, prob.quad
        x, w = oracle.gauss(q)
        self.L = np.array([[oracle.legendre(i, xa) for i in range(n)] for xa in x])  # [a][i]
        self.w = w
        h = (prob.upper - prob.lower) / prob.cells
        self.detK = float(np.prod(h))
        self.n, self.q = n, q
        # Phi[abc, ijk] = L_i(x_a) L_j(x_b) L_k(x_c); W[abc] = w_a w_b w_c |K|
        self.Phi = np.einsum("ai,bj,ck->abcijk", self.L, self.L, self.L).reshape(q ** 3, n ** 3)
        self.W = np.einsum("a,b,c->abc", w, w, w).ravel() * self.detK
        # physical coordinates of every cell's points [cell][abc] (cell = ix + Nx (iy + Ny iz))
        nx, ny, nz = (int(c) for c in prob.cells)
        iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()
        A, B, Cc = np.meshgrid(x, x, x, indexing="ij")
        self.X = prob.lower[0] + (ix[:, None] + A.ravel()[None, :]) * h[0]
        self.Y = prob.lower[1] + (iy[:, None] + B.ravel()[None, :]) * h[1]
        self.Z = prob.lower[2] + (iz[:, None] + Cc.ravel()[None, :]) * h[2]

    def r(self, u):
        if self.user:
            return self.ufun(u, self.X, self.Y, self.Z)
        return self.c1 * u + self.c3 * u ** 3 + self.ce * np.exp(u)

    def dr(self, u):
        if self.user:
            return self.udfun(u, self.X, self.Y, self.Z)
        return self.c1 + 3.0 * self.c3 * u ** 2 + self.ce * np.exp(u)

    def _points(self, u):
        return np.asarray(u, dtype=np.float64).reshape(-1, self.n ** 3) @ self.Phi.T  # [cell][abc]

    def reaction(self, u):
        return ((self.W * self.r(self._points(u))) @ self.Phi).ravel()

    def apply(self, u):
        return self.prob.apply(u) + self.reaction(u)

    def jacobian_apply(self, u0, d):
        c = self.W * self.dr(self._points(u0))
        return self.prob.apply(d) + ((c * self._points(d)) @ self.Phi).ravel()

    def jacobian_blocks(self, u0):
        """Element-diagonal blocks of the Jacobian at u0: [cell][i][j]."""
        c = self.W * self.dr(self._points(u0))  # [cell][abc]
        react = np.einsum("zp,pi,pj->zij", c, self.Phi, self.Phi)
        return self.prob.block_diagonal() + react

    def jacobian_matrix(self, u0):
        nd = self.prob.ndofs
        return np.stack([self.jacobian_apply(u0, e) for e in np.eye(nd)], axis=1)


SUCCESS, INVALID_RESIDUAL, LINE_SEARCH_FAILED, TOO_MANY_ITERATIONS, TOO_MANY_LINEAR_ITERATIONS, LINEAR_SOLVER_FAILED = (
    0, 1, 4, 5, 6, 7)


def newton(S, jacobian_solve, rhs, w, tolerance=1e-6, max_iterations=2 ** 31 - 1, max_linear_iterations=2 ** 31 - 1,
           line_search=False, max_line_search_iterations=2 ** 31 - 1, forcing=False, eta_max=0.99, gamma=0.1):
    """Newton for S(w) = rhs.  jacobian_solve(w, r, lin_tol) -> (dw, linear iterations, negative if failed).
    Returns (w, info dict) with the reference's counters and failure code."""
    w = np.array(w, dtype=np.float64)
    st = {"it": 0, "lin": 0, "done": True, "delta": 0.0, "prev_eta": -1.0, "prev_res": -1.0, "lin_tol": None,
          "halvings": 0, "history": []}

    def failed():
        d = st["delta"]
        if not (d < np.finfo(np.float64).max) or math.isnan(d):
            return INVALID_RESIDUAL
        if st["it"] >= max_iterations:
            return TOO_MANY_ITERATIONS
        if st["lin"] >= max_linear_iterations:
            return TOO_MANY_LINEAR_ITERATIONS
        if st["lin"] < 0:
            return LINEAR_SOLVER_FAILED
        if not st["done"]:
            return LINE_SEARCH_FAILED
        return SUCCESS

    def update_linear_tolerance():
        if not forcing:
            return
        cur = st["delta"]
        eta = eta_max
        if st["prev_eta"] >= 0.0:
            eta_a = gamma * cur * cur / (st["prev_res"] * st["prev_res"])
            ind = gamma * st["prev_eta"] ** 2
            eta_c = min(eta_a, eta_max) if ind < 0.1 else min(eta_max, max(eta_a, ind))
            eta = min(eta_max, max(eta_c, 0.5 * tolerance / cur))
        st["prev_res"], st["prev_eta"] = cur, eta
        st["lin_tol"] = eta

    def norm(v):
        return math.sqrt(float(np.dot(v, v)))

    residual = S(w) - rhs
    st["delta"] = norm(residual)
    update_linear_tolerance()
    while True:
        if max_linear_iterations - st["lin"] <= 0:
            break
        dw, its = jacobian_solve(w, residual, st["lin_tol"])
        if its < 0:
            st["lin"] = its
            break
        st["lin"] += its
        w = w - dw
        residual = S(w) - rhs
        # line search
        delta_old = st["delta"]
        st["delta"] = norm(residual)
        ls = 0
        if line_search:
            if failed() == INVALID_RESIDUAL:
                t = float(np.dot(dw, dw))
                if not (t < np.finfo(np.float64).max and not math.isnan(t)):
                    st["delta"] = 2.0 * delta_old
            factor = 1.0
            ls = 1 if st["delta"] < delta_old else 0
            k = 0
            while st["delta"] >= delta_old:
                delta_prev = st["delta"]
                factor *= 0.5
                if abs(st["delta"] - delta_old) < 1e-5 * st["delta"]:
                    ls = -1
                    break
                w = w + factor * dw
                st["halvings"] += 1
                residual = S(w) - rhs
                st["delta"] = norm(residual)
                if abs(st["delta"] - delta_prev) < 1e-15:
                    ls = -1
                    break
                if failed() == INVALID_RESIDUAL:
                    st["delta"] = 2.0 * delta_old
                k += 1
                if k >= max_line_search_iterations:
                    ls = -1
                    break
        st["done"] = ls >= 0
        update_linear_tolerance()
        st["it"] += 1
        st["history"].append(st["delta"])
        if st["delta"] < tolerance or failed() != SUCCESS:
            break
    return w, {"iterations": st["it"], "linear_iterations": st["lin"], "residual": st["delta"],
               "failure": failed(), "converged": failed() == SUCCESS, "line_search_halvings": st["halvings"],
               "residuals": st["history"]}
