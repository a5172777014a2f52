"""dune.fem-shaped scheme construction from UFL-shaped forms:
galerkin([a == b, DirichletBC(space, g)], solver=...) on dglegendre spaces
(python/dune/fem/scheme/__init__.py), compiled at run time."""
import numpy as np
import pytest


def _problem():
    """-div((1 + u^2) grad u) + u = sin(pi x) y on the unit cube, u = x y + 1/2
    weakly on the boundary; DG Q2 on 4^3 cells."""
    import ufl_forms as U
    space = U.dglegendre((4, 4, 4), 2)
    u, v, x = U.TrialFunction(1), U.TestFunction(1), U.SpatialCoordinate()
    a = ((1 + u[0] ** 2) * U.inner(U.grad(u)[0, :], U.grad(v)[0, :]) + u[0] * v[0]) * U.dx
    b = U.sin(np.pi * x[0]) * x[1] * v[0] * U.dx
    bc = U.DirichletBC(space, x[0] * x[1] + 0.5)
    return U, space, a, b, bc


def test_equation_and_argument_checks():
    U, space, a, b, bc = _problem()
    eq = a == b
    assert isinstance(eq, U.Equation)
    r = eq.residual()
    assert ("v", 0) in r.terms and ("g", 0, 0) in r.terms
    assert (a == 0).residual() is a
    with pytest.raises(ValueError):
        U.galerkin([a == b, a == 0], space)
    with pytest.raises(ValueError):
        U.galerkin(a == b)  # no space
    u, v = U.TrialFunction(1), U.TestFunction(1)
    faces = a + (u[0] * v[0]) * U.ds
    with pytest.raises(ValueError):
        U.galerkin([faces == 0, bc])  # boundary terms given twice
    with pytest.raises(ValueError):
        U.galerkin([a == b, U.DirichletBC(space, [0.0, 1.0])])  # two values for one component


@pytest.mark.gpu
def test_galerkin_scheme_solves_the_discrete_problem(gb):
    """scheme.solve reaches a w whose residual in the form oracle's operator
    (the same SIPG form, evaluated independently on the CPU) is at the
    tolerance."""
    import form_oracle as fo
    U, space, a, b, bc = _problem()
    scheme = U.galerkin([a == b, bc], solver="gmres",
                        parameters={"nonlinear.tolerance": 1e-10, "linear.tolerance": 1e-12,
                                    "linear.gmres.restart": 60, "linear.preconditioning.method": "blockjacobi"})
    w = space.zero
    info = scheme.solve(target=w)
    assert info["converged"] and info["iterations"] >= 2, info

    def flux(x, u, g):
        return (1.0 + u[:, :, None] ** 2) * g

    def source(x, u, g):
        return u - (np.sin(np.pi * x[:, 0]) * x[:, 1])[:, None]

    I, S, B = fo.sipg(1, flux=flux, source=source, dirichlet=lambda x: (x[:, 0] * x[:, 1] + 0.5)[:, None])
    spec = fo.FormSpec(space.cells, space.order, 1, I, S, B)
    wn = w.numpy()
    res = fo.residual(spec, wn)
    assert np.linalg.norm(res) < 1e-9
    # and the scheme's own operator agrees with the oracle at the solution
    # (both near zero: rounding of terms of size ~penalty / h)
    y = space.zero
    scheme(w, y)
    assert np.max(np.abs(y.numpy() - res)) < 1e-10
