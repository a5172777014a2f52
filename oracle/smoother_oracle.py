"""Oracle of the stationary-iteration preconditioners on an assembled matrix.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker; the product never
imports it.

Restates FemPreconditioningBase::apply (solver/fempreconditioning.hh:130-161)
and SparseRowMatrix::doParallelIterative (operator/matrix/spmatrix.hh:446-480)
on a dense matrix: rows in natural order (reverse for the backward sweep),
x_i = w (b_i - sum_{j != i} a_ij x_j) / a_ii, x read from the vector being
written (Gauss-Seidel, SOR, SSOR) or from the previous iterate (Jacobi),
starting from x = 0.
"""
import numpy as np


def smoother_apply(A, b, method="ssor", iterations=1, relaxation=1.0):
    A = np.asarray(A, dtype=np.float64)
    n = A.shape[0]
    d = np.diag(A).copy()
    eps = 16.0 * np.finfo(np.float64).eps
    dinv = np.where(np.abs(d) < eps, 1.0, 1.0 / np.where(np.abs(d) < eps, 1.0, d))
    w = 1.0 if method == "gauss-seidel" else relaxation
    v = np.zeros(n)
    xtmp = np.zeros(n)

    def sweep(xold, xnew, forward):
        rows = range(n) if forward else range(n - 1, -1, -1)
        for i in rows:
            rhs = b[i]
            for j in np.nonzero(A[i])[0]:
                if j != i:
                    rhs -= A[i, j] * xold[j]
            xnew[i] = w * (rhs * dinv[i])

    for it in range(iterations):
        if method == "jacobi":
            sweep(xtmp, v, True)
            if it < iterations - 1:
                xtmp = v.copy()
        else:
            sweep(v, v, True)
            if method == "ssor":
                sweep(v, v, False)
    return v
