"""Newton's method against dune-fem's own NewtonInverseOperator.

tests/golden/ref_newton.json was made by oracle/make_ref_golden.sh, which
compiles the reference's solver/newtoninverseoperator.hh unmodified (its
NewtonParameter, line search and stopping rule) and runs it on S(w) = f,
S the reference's DGEllipticOperator with the source r(u) = c1 u + c3 u^3 +
ce exp(u) and its Jacobian from DifferentiableDGEllipticOperator::jacobian,
each Newton step solved exactly (dense LU).  The golden vectors hold the
residual norm after every step, the step counts and the solution, for a
cubic reaction with a kappa field (also with the Eisenstat-Walker forcing,
whose linear tolerances the golden vectors record), an exponential one, and
an Allen-Cahn problem started near its inflection point without and with the
line search.
"""
import json
import os

import numpy as np
import pytest

from conftest import relmax

with open(os.path.join(os.path.dirname(__file__), "golden", "ref_newton.json")) as _f:
    CASES = {c["name"]: c for c in json.load(_f)["cases"]}


def setup(case):
    """The right-hand side, initial guess and kappa field of a case, rebuilt
    exactly from the driver's integer formulas."""
    p = case["order"]
    nl = (p + 1) ** 3
    ncell = int(np.prod(case["cells"]))
    i = np.arange(ncell * nl, dtype=np.int64)
    f = case["rhs_scale"] * (((i * 7919 + 13) % 2003 - 1001) / 1000.0)
    w0 = np.zeros(ncell * nl)
    w0[::nl] = case["w0_constant"]
    kappa = None
    if case["kappa_field"]:
        c = np.arange(ncell, dtype=np.int64)
        idx = c[:, None] * nl + np.arange(nl, dtype=np.int64)[None, :]
        kappa = ((idx * 37 + 5) % 9 - 4) / 1000.0
        kappa[:, 0] = 1.0 + ((c * 31 + 7) % 11) / 10.0
        kappa = kappa.reshape(-1)
    return f, w0, kappa


def operator_kw(case):
    return dict(quad_points=case["quad_points"], diffusion=case["diffusion"], penalty=case["penalty"],
                periodic=tuple(case["periodic"]), weak_dirichlet=False)


def test_golden_cases():
    assert set(CASES) == {"cubic_periodic_kappa", "cubic_periodic_kappa_eisenstat_walker", "exp_periodic",
                          "allen_cahn_plain", "allen_cahn_line_search"}
    assert all(c["converged"] for c in CASES.values())
    # the line search shortens the Allen-Cahn solve
    assert CASES["allen_cahn_line_search"]["iterations"] < CASES["allen_cahn_plain"]["iterations"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_newton_equals_reference(orc, name):
    """The restated Newton loop (oracle/nonlinear_oracle.py) over the oracle's
    operator and reaction, with exact linear solves: the same number of steps,
    the same residual after every step and the same solution."""
    import nonlinear_oracle as no
    case = CASES[name]
    f, w0, kappa = setup(case)
    prob = orc.DGProblem(tuple(case["cells"]), case["order"], **operator_kw(case))
    P = no.NonlinearProblem(prob, tuple(case["reaction"]))
    n, nl = prob.ndofs, prob.nloc
    A = np.stack([prob.apply(e, kappa=kappa) for e in np.eye(n)], axis=1)

    def S(w):
        return A @ w + P.reaction(w)

    def jacobian(w):
        c = P.W * P.dr(P._points(w))
        blocks = np.einsum("zp,pi,pj->zij", c, P.Phi, P.Phi)
        J = A.copy()
        for z in range(prob.ncells):
            J[z * nl:(z + 1) * nl, z * nl:(z + 1) * nl] += blocks[z]
        return J

    forcing = case["forcing"] == "eisenstatwalker"
    tolerances = []

    def solve(w, r, tol):
        tolerances.append(tol)
        return np.linalg.solve(jacobian(w), r), 1

    w, info = no.newton(S, solve, f, w0, tolerance=case["tolerance"], line_search=case["line_search"] == "simple",
                        forcing=forcing)
    assert info["converged"]
    assert info["iterations"] == case["iterations"] and info["linear_iterations"] == case["linear_iterations"]
    scale = max(case["initial_residual"], float(np.linalg.norm(f)))
    for got, ref in zip(info["residuals"], case["residuals"]):
        assert abs(got - ref) <= 1e-9 * ref + 1e-13 * scale
    assert relmax(w, case["w"]) < 1e-12
    if forcing:
        # the forcing terms follow the residuals; the last ones are taken from
        # residuals at the rounding floor
        assert len(tolerances) == len(case["linear_tolerances"])
        for k, (got, ref) in enumerate(zip(tolerances, case["linear_tolerances"])):
            if k == 0 or case["residuals"][k - 1] > 1e3 * case["tolerance"]:
                assert abs(got - ref) <= 1e-9 * ref


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if c["forcing"] == "none"))
def test_gpu_newton_equals_reference(gb, name):
    """NewtonInverseOperator over NonlinearDGOperator on the GPU: the same
    number of Newton steps and the same solution as the reference's Newton.
    The Jacobian systems are solved by CG (SPD cases) or full GMRES (the
    indefinite Allen-Cahn Jacobians) to 1e-13, not exactly."""
    case = CASES[name]
    f, w0, kappa = setup(case)
    op = gb.NonlinearDGOperator(tuple(case["cells"]), case["order"], reaction=tuple(case["reaction"]),
                                kappa=None if kappa is None else gb.DeviceArray.from_numpy(kappa),
                                **operator_kw(case))
    indefinite = case["reaction"][0] < 0
    newton = gb.NewtonInverseOperator(tolerance=case["tolerance"], line_search=case["line_search"],
                                      linear_method="gmres" if indefinite else "cg", linear_tolerance=1e-13,
                                      linear_restart=200, linear_max_iterations=10000,
                                      max_linear_iterations=10 ** 6, max_iterations=100,
                                      preconditioner=gb.PC_BLOCK_JACOBI)
    newton.bind(op)
    w = gb.DeviceArray.from_numpy(w0)
    newton(gb.DeviceArray.from_numpy(f), w)
    info = newton.info()
    assert info["converged"], info
    assert info["iterations"] == case["iterations"], info
    assert info["residual"] < case["tolerance"]
    assert relmax(w.numpy(), case["w"]) < 1e-9
