"""The coefficient-space ("closed form") SIPG/upwind apply, restated in numpy
exactly as the CUDA kernels organise it, against the oracle's Gauss-point
apply (no GPU).

The CUDA path (dune-fem_gb300/csrc/dg_const_kernel.cuh) does not integrate at
Gauss points: for constant (or cellwise constant) kappa on affine cells with
the orthonormal Legendre basis the integrands are polynomials that the rule
integrates exactly, so the apply can be written with 1-D line operators and
face traces.  The kernel folds the flux constants:
  - traces per face s of every cell: v(s) = sum_i L_i(s) u_i and
    P(s) = v(s) - sigma_s r dv(s) (r = A2 / C; kappa per cell: P = sigma_s dv);
  - interior flux Val / C = P- - P+ + (A1/C - 1) J and Grad / (-A2) = J;
  - C and -A2 in the per-axis expansion tables.
This restatement checks that algebra (signs, the boundary and upwind terms,
the A1 = 0 cases) against the oracle, which follows the reference's
GalerkinOperator (schemes/galerkin.hh:332-537) with the SIPG form of
pydemo/advectiondiffusion.py:33-55.
"""
import numpy as np
import pytest

from conftest import relmax


def _legendre(k, x, deriv=False):
    c = np.zeros(k + 1)
    c[k] = 1.0
    if deriv:
        return 2.0 * np.sqrt(2 * k + 1) * np.polynomial.legendre.legval(2 * x - 1, np.polynomial.legendre.legder(c))
    return np.sqrt(2 * k + 1) * np.polynomial.legendre.legval(2 * x - 1, c)


def closed_form_apply(cells, p, eps, pen, mass, vel, weak_dirichlet, periodic, u, kcell=None):
    n = p + 1
    h = [1.0 / c for c in cells]
    vol = float(np.prod(h))
    xg, wg = np.polynomial.legendre.leggauss(n + 1)
    xg, wg = (xg + 1) / 2, wg / 2
    dL = np.array([[_legendre(i, x, True) for x in xg] for i in range(n)])
    Lv = np.array([[_legendre(i, x) for x in xg] for i in range(n)])
    K1 = (dL * wg) @ dL.T            # int L_i' L_j'
    D1 = (dL * wg) @ Lv.T            # int L_i' L_j
    L1 = np.array([_legendre(i, 1.0) for i in range(n)])
    dL1 = np.array([_legendre(i, 1.0, True) for i in range(n)])
    sgn = (-1.0) ** np.arange(n)     # L_i(0) = (-1)^i L_i(1)
    kc = kcell is not None
    aC = 1.0 if eps * pen != 0.0 else 0.0
    U = u.reshape(cells[2], cells[1], cells[0], n, n, n)  # [cz][cy][cx][i0][i1][i2]
    W = np.zeros_like(U)
    K = None if kcell is None else kcell.reshape(cells[2], cells[1], cells[0])[..., None, None]
    cell_axis = {0: 2, 1: 1, 2: 0}

    def lines(A, d):  # the degree along axis d last
        return np.moveaxis(A, 3 + d, -1)

    for d in range(3):
        area = vol / h[d]
        A1 = area * eps * pen / h[d]
        A2 = area * eps * 0.5 / h[d]
        C = A1 if aC else 1.0
        pc = dL1 if kc else L1 - (A2 / C) * dL1
        X = lines(U, d)
        V = {1: X @ L1, 0: X @ (sgn * L1)}
        P = {1: X @ pc, 0: X @ (sgn * pc)}
        ax, N = cell_axis[d], cells[d]
        val, grad = {}, {}
        for s in (0, 1):
            step = 1 if s else -1
            vm, pm = V[s], P[s]
            vp = np.roll(V[1 - s], -step, axis=ax)
            pp = np.roll(P[1 - s], -step, axis=ax)
            nb = np.arange(N) + step
            has = ((nb >= 0) & (nb < N)) | bool(periodic[d])
            shape = [1] * 5
            shape[ax] = N
            has = has.reshape(shape)
            bn = vel[d] if s else -vel[d]
            J = vm - vp
            if kc:
                kp = np.roll(K, -step, axis=ax)
                vi = A1 * 0.5 * (K + kp) * J - A2 * (K * pm - kp * pp)
                gi = -A2 * K * J
                vb = A1 * K * vm - 2 * A2 * K * pm if weak_dirichlet else 0 * vm
                gb = -2 * A2 * K * vm if weak_dirichlet else 0 * vm
            else:
                vi = pm - pp + (aC - 1.0) * J + (area * bn / C) * (vm if bn >= 0 else vp)
                gi = J
                vb = (aC - 2.0) * vm + 2 * pm if weak_dirichlet else 0 * vm
                gb = 2 * vm if weak_dirichlet else 0 * vm
                if bn > 0:
                    vb = vb + (area * bn / C) * vm
            val[s], grad[s] = np.where(has, vi, vb), np.where(has, gi, gb)
        vs, vd = val[1] + val[0], val[1] - val[0]
        gs, gd = grad[1] + grad[0], grad[1] - grad[0]
        M = eps * vol / h[d] ** 2 * K1 - vel[d] * vol / h[d] * D1
        if kc:
            Y = (X @ M.T) * K[..., None]
            if d == 0:
                Y = Y + mass * vol * X
            et, edt = L1, dL1
        else:
            if d == 0:
                M = M + mass * vol * np.eye(n)
            Y = X @ M.T
            et, edt = C * L1, -A2 * dL1
        E = np.stack([et[i] * (vd if i & 1 else vs) + edt[i] * (gd if i & 1 else gs) for i in range(n)], -1)
        lines(W, d)[...] += Y + E
    return W.reshape(-1)


CASES = {
    "sipg_q3": ((3, 4, 5), 3, dict(diffusion=1.0, penalty=160.0)),
    "mass_periodic_q2": ((3, 4, 5), 2, dict(diffusion=0.7, penalty=90.0, mass=0.3, periodic=(1, 0, 1))),
    "advection_diffusion_periodic": ((4, 3, 3), 2, dict(diffusion=1e-3, penalty=90.0, velocity=(1.0, 0.5, 0.25),
                                                        periodic=(1, 1, 1))),
    "advection_boundaries_q3": ((4, 3, 3), 3, dict(diffusion=1e-3, penalty=160.0, velocity=(1.0, -0.5, 0.25))),
    "pure_advection": ((4, 3, 3), 1, dict(diffusion=0.0, penalty=40.0, velocity=(1.0, -0.5, 0.25),
                                          weak_dirichlet=False, periodic=(0, 1, 0))),
    "no_penalty": ((3, 3, 4), 2, dict(diffusion=1.0, penalty=0.0, mass=0.2, periodic=(0, 0, 1))),
    "q4_no_weak_dirichlet": ((3, 3, 4), 4, dict(diffusion=1.0, penalty=250.0, weak_dirichlet=False)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_folded_closed_form_matches_the_oracle(orc, case):
    cells, p, kw = CASES[case]
    prob = orc.DGProblem(cells, p, **kw)
    u = np.random.default_rng(1).uniform(-1, 1, prob.ndofs)
    w = closed_form_apply(cells, p, kw.get("diffusion", 1.0), kw["penalty"], kw.get("mass", 0.0),
                          kw.get("velocity", (0.0, 0.0, 0.0)), kw.get("weak_dirichlet", True),
                          kw.get("periodic", (0, 0, 0)), u)
    assert relmax(w, prob.apply(u)) < 1e-12


@pytest.mark.parametrize("p,periodic,mass", [(3, (0, 0, 0), 0.0), (2, (0, 1, 0), 0.5)])
def test_folded_closed_form_with_cellwise_kappa(orc, p, periodic, mass):
    """kappa constant per cell: the oracle integrates kappa as a DG field whose
    only nonzero coefficient is the cell mean."""
    cells = (3, 4, 5)
    prob = orc.DGProblem(cells, p, penalty=10.0 * (p + 1) ** 2, mass=mass, periodic=periodic)
    rng = np.random.default_rng(2)
    u = rng.uniform(-1, 1, prob.ndofs)
    kcell = np.exp(rng.normal(size=prob.ncells))
    kappa = np.zeros((prob.ncells, prob.nloc))
    kappa[:, 0] = kcell
    w = closed_form_apply(cells, p, 1.0, prob.penalty, mass, (0.0, 0.0, 0.0), True, periodic, u, kcell)
    assert relmax(w, prob.apply(u, kappa=kappa.reshape(-1))) < 1e-12
