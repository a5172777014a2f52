"""Convergence order of the DG form, as the reference's own demo checks it
(pydemo/advectiondiffusion.py:104-106: the L2 EOC of DG P2 with SIPG diffusion
and upwind advection is at least p + 1 - 0.1).

On the CPU with the oracle, which the GPU operator matches to 1e-12 (the
parity tests), so the order pins the form itself: a sign or scaling slip in
any face term would cost convergence.  Manufactured solution
u = sin(pi x) sin(pi y) sin(pi z) on the unit cube (u = 0 on the boundary,
weak Dirichlet), -eps Lap u + b.grad u = f, block-Jacobi-preconditioned
GMRES(30) to 1e-12.
"""
import numpy as np
import pytest

EPS = 1.0
B = (1.0, 0.5, 0.25)


def _basis(n, x):
    """Orthonormal Legendre on [0, 1] at the points x: [len(x)][n]."""
    out = np.empty((len(x), n))
    for i in range(n):
        c = np.zeros(i + 1)
        c[i] = 1.0
        out[:, i] = np.sqrt(2 * i + 1) * np.polynomial.legendre.legval(2 * x - 1, c)
    return out


def _rule(q):
    x, w = np.polynomial.legendre.leggauss(q)
    return (x + 1) / 2, w / 2


def _load_vector(N, p):
    """b_l = int f phi_l, f = 3 pi^2 eps u + b.grad u: four separable terms,
    each a tensor product of 1-D cell integrals."""
    n, h = p + 1, 1.0 / N
    xq, wq = _rule(p + 3)
    Bq = _basis(n, xq)
    pts = (np.arange(N)[:, None] + xq[None, :]) * h          # [cell][point]
    s, c = np.sin(np.pi * pts), np.cos(np.pi * pts)
    Is = h * np.einsum("ca,a,ai->ci", s, wq, Bq)               # int sin(pi x) phi_i over each cell
    Ic = h * np.einsum("ca,a,ai->ci", c, wq, Bq)
    terms = [(3 * np.pi ** 2 * EPS, Is, Is, Is), (np.pi * B[0], Ic, Is, Is), (np.pi * B[1], Is, Ic, Is),
             (np.pi * B[2], Is, Is, Ic)]
    b = sum(k * np.einsum("xi,yj,zk->zyxijk", gx, gy, gz) for k, gx, gy, gz in terms)
    return b.reshape(-1)


def _l2_error(N, p, uh):
    n, h = p + 1, 1.0 / N
    xq, wq = _rule(p + 3)
    Bq = _basis(n, xq)
    U = uh.reshape(N, N, N, n, n, n)                            # [cz][cy][cx][i0][i1][i2]
    vals = np.einsum("zyxijk,ai,bj,ck->zyxabc", U, Bq, Bq, Bq)  # a: x point, b: y, c: z
    pts = (np.arange(N)[:, None] + xq[None, :]) * h
    s = np.sin(np.pi * pts)
    exact = np.einsum("xa,yb,zc->zyxabc", s, s, s)
    w3 = np.einsum("a,b,c->abc", wq, wq, wq)
    return np.sqrt(np.sum((vals - exact) ** 2 * w3) * h ** 3)


def _solve(orc, N, p):
    prob = orc.DGProblem((N, N, N), p, diffusion=EPS, velocity=B)
    blocks = np.linalg.inv(prob.block_diagonal(nthreads=8))
    nloc = prob.nloc
    op = lambda x: prob.apply(x, nthreads=8)
    prec = lambda r: np.einsum("cij,cj->ci", blocks, r.reshape(-1, nloc)).reshape(-1)
    it, x, res = orc.gmres(op, _load_vector(N, p), 30, prec=prec, tolerance=1e-12, max_iter=3000)
    assert it >= 0, "GMRES did not converge (residual %g)" % res
    return _l2_error(N, p, x)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_sipg_upwind_l2_order(orc, p):
    """Measured: EOC 2.00, 2.97, 3.97 for p = 1, 2, 3 between 4^3 and 8^3."""
    errs = [_solve(orc, N, p) for N in (4, 8)]
    eoc = np.log(errs[0] / errs[1]) / np.log(2.0)
    assert eoc >= p + 1 - 0.1, (errs, eoc)


def _q1_solve_error(orc, N):
    """Config 1's form: -Lap u + u = f on the unit square, continuous Q1,
    u = sin(pi x) sin(pi y) (zero on the boundary), diagonal-preconditioned CG."""
    h = 1.0 / N
    xq, wq = _rule(3)
    pts = (np.arange(N)[:, None] + xq[None, :]) * h           # [cell][point]
    s = np.sin(np.pi * pts)
    hat = np.stack([1 - xq, xq], 1)                            # [point][k]
    I = h * np.einsum("ca,a,ak->ck", s, wq, hat)               # int sin(pi x) phi_k over each cell
    S = np.zeros(N + 1)                                        # int sin(pi x) phi_v over [0, 1]
    S[:-1] += I[:, 0]
    S[1:] += I[:, 1]
    b = (2 * np.pi ** 2 + 1) * np.outer(S, S).reshape(-1)      # vertex v = vy (N + 1) + vx
    edge = np.zeros((N + 1, N + 1), bool)
    edge[0, :] = edge[-1, :] = edge[:, 0] = edge[:, -1] = True
    b[edge.reshape(-1)] = 0.0                                  # Dirichlet rows: u_D = g = 0
    cells = (N, N)
    diag = orc.q1_apply(cells, None, 1.0, 1.0, diag_only=True)
    it, x, res = orc.cg(lambda v: orc.q1_apply(cells, v, 1.0, 1.0), b, prec=lambda r: r / diag,
                        epsilon=1e-12, max_iter=5000)
    assert it >= 0, "CG did not converge (residual %g)" % res
    U = x.reshape(N + 1, N + 1)                                # [vy][vx]
    # bilinear u_h at the Gauss points of every cell: [cy][cx][b][a]
    vals = sum(np.einsum("yx,b,a->yxba", U[ky:ky + N, kx:kx + N], hat[:, ky], hat[:, kx])
               for ky in (0, 1) for kx in (0, 1))
    exact = np.einsum("yb,xa->yxba", s, s)
    return np.sqrt(np.sum((vals - exact) ** 2 * np.outer(wq, wq)) * h * h)


def test_q1_l2_order(orc):
    """Measured: L2 EOC 2.00 between 16^2 and 32^2."""
    errs = [_q1_solve_error(orc, N) for N in (16, 32)]
    eoc = np.log(errs[0] / errs[1]) / np.log(2.0)
    assert eoc >= 2 - 0.1, (errs, eoc)
