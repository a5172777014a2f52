"""Nonlinear DG operator S(u) = A u + int r(u) v, its Jacobian and Newton's
method (NewtonInverseOperator), on the GPU through the C-ABI, against the
oracle (oracle/nonlinear_oracle.py)."""
import numpy as np
import pytest

from conftest import relmax

TOL64 = 1e-12


def _no():
    import nonlinear_oracle
    return nonlinear_oracle


# ---------------------------------------------------------------- CPU tests --
def test_oracle_linear_reaction_is_the_mass_matrix(orc):
    """r(u) = c u: with the orthonormal basis and q >= p+1 the reaction is c |K| u."""
    no = _no()
    prob = orc.DGProblem((2, 3, 2), 2, lower=(0, 0, 0), upper=(1.0, 1.5, 0.5))
    P = no.NonlinearProblem(prob, (0.7, 0.0, 0.0))
    u = np.random.default_rng(1).uniform(-1, 1, prob.ndofs)
    vol = 1.0 / 2 * 1.5 / 3 * 0.5 / 2
    assert relmax(P.reaction(u), 0.7 * vol * u) < 1e-13


def test_oracle_jacobian_is_the_derivative(orc):
    no = _no()
    prob = orc.DGProblem((2, 2, 2), 1, mass=0.3)
    P = no.NonlinearProblem(prob, (0.5, 2.0, -0.3))
    rng = np.random.default_rng(2)
    u, d = rng.uniform(-1, 1, prob.ndofs), rng.uniform(-1, 1, prob.ndofs)
    eps = 1e-5
    fd = (P.apply(u + eps * d) - P.apply(u - eps * d)) / (2 * eps)
    assert relmax(P.jacobian_apply(u, d), fd) < 1e-8
    J = P.jacobian_matrix(u)
    blocks = P.jacobian_blocks(u)
    nl = prob.nloc
    for c in range(prob.ncells):
        assert relmax(blocks[c], J[c * nl:(c + 1) * nl, c * nl:(c + 1) * nl]) < 1e-12


def test_oracle_newton_is_quadratic_and_line_search_cuts_steps(orc):
    no = _no()
    prob = orc.DGProblem((3, 3, 3), 1)
    P = no.NonlinearProblem(prob, (0.0, 0.0, -5.0))  # Bratu: -lap u = 5 e^u
    rhs = np.zeros(prob.ndofs)
    solve = lambda w, r, tol: (np.linalg.solve(P.jacobian_matrix(w), r), 1)
    w, info = no.newton(P.apply, solve, rhs, np.zeros(prob.ndofs), tolerance=1e-10)
    assert info["converged"] and info["iterations"] == 3 and info["residual"] < 1e-10
    # Allen-Cahn-type r = u^3 - u from near the inflection: the full steps
    # overshoot, the line search halves them and Newton needs fewer steps
    prob2 = orc.DGProblem((2, 2, 2), 1, diffusion=1e-3)
    P2 = no.NonlinearProblem(prob2, (-1.0, 1.0, 0.0))
    w0 = prob2.project(2, params=(0.58,))
    s2 = lambda w, r, tol: (np.linalg.solve(P2.jacobian_matrix(w), r), 1)
    _, i_plain = no.newton(P2.apply, s2, np.zeros(prob2.ndofs), w0, tolerance=1e-10)
    _, i_ls = no.newton(P2.apply, s2, np.zeros(prob2.ndofs), w0, tolerance=1e-10, line_search=True)
    assert i_ls["converged"] and i_ls["line_search_halvings"] > 0 and i_ls["iterations"] < i_plain["iterations"]


# ---------------------------------------------------------------- GPU tests --
@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("reaction", [(0.0, 1.5, 0.0), (0.3, 0.0, -0.8), (-1.0, 1.0, 0.2)])
@pytest.mark.parametrize("algorithm", [0, 1])
def test_nonlinear_apply_matches_oracle(gb, orc, order, reaction, algorithm):
    no = _no()
    cells = (3, 2, 4)
    kw = dict(mass=0.4, velocity=(0.5, 0.0, -0.25), periodic=(0, 1, 0), lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction, algorithm=algorithm, **kw)
    assert op.nonlinear()
    P = no.NonlinearProblem(orc.DGProblem(cells, order, **kw), reaction)
    u = np.random.default_rng(30 + order).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), P.apply(u)) < TOL64


@pytest.mark.gpu
def test_nonlinear_apply_fp32(gb, orc):
    no = _no()
    cells, order, reaction = (3, 3, 3), 2, (0.2, 1.0, -0.5)
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction, precision=gb.F32)
    P = no.NonlinearProblem(orc.DGProblem(cells, order), reaction)
    u = np.random.default_rng(3).uniform(-1, 1, op.size).astype(np.float32)
    w = gb.DeviceArray(op.size, gb.F32)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), P.apply(u.astype(np.float64))) < 2e-5


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 3])
def test_jacobian_apply_diagonal_and_blocks_match_oracle(gb, orc, order):
    no = _no()
    cells, reaction = (3, 2, 2), (0.4, 2.0, -0.6)
    kw = dict(mass=0.2, velocity=(0.3, -0.2, 0.1))
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction, **kw)
    P = no.NonlinearProblem(orc.DGProblem(cells, order, **kw), reaction)
    rng = np.random.default_rng(40 + order)
    u0, d = rng.uniform(-1, 1, op.size), rng.uniform(-1, 1, op.size)
    jac = op.jacobian(gb.DeviceArray.from_numpy(u0))
    assert not jac.nonlinear()
    y = gb.DeviceArray(op.size)
    jac(gb.DeviceArray.from_numpy(d), y)
    assert relmax(y.numpy(), P.jacobian_apply(u0, d)) < TOL64
    nl = op.nloc
    blocks = jac.block_diagonal(nl).numpy().reshape(-1, nl, nl)
    ref = P.jacobian_blocks(u0)
    assert relmax(blocks, ref) < TOL64
    assert relmax(jac.diagonal().numpy(), np.einsum("cii->ci", ref).ravel()) < TOL64
    # re-linearising the same Jacobian object at another point
    u1 = rng.uniform(-1, 1, op.size)
    op.jacobian(gb.DeviceArray.from_numpy(u1), jac)
    jac(gb.DeviceArray.from_numpy(d), y)
    assert relmax(y.numpy(), P.jacobian_apply(u1, d)) < TOL64
    # the assembled Jacobian reproduces the matrix-free one
    A = jac.assemble()
    ya = gb.DeviceArray(op.size)
    A(gb.DeviceArray.from_numpy(d), ya)
    assert relmax(ya.numpy(), y.numpy()) < 1e-13
    # a nonlinear operator has no matrix of its own
    with pytest.raises(gb.GbfemError):
        op.diagonal()


@pytest.mark.gpu
def test_newton_bratu_matches_oracle_newton(gb, orc):
    """-lap u = 5 e^u (SIPG, weak u = 0): quadratic convergence, the same
    Newton iterations as the oracle's restated loop with exact linear solves."""
    no = _no()
    cells, order, reaction = (3, 3, 3), 2, (0.0, 0.0, -5.0)
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction)
    P = no.NonlinearProblem(orc.DGProblem(cells, order), reaction)
    solve = lambda w, r, tol: (np.linalg.solve(P.jacobian_matrix(w), r), 1)
    wo, io = no.newton(P.apply, solve, np.zeros(op.size), np.zeros(op.size), tolerance=1e-10)
    for pc in (gb.PC_BLOCK_JACOBI, gb.PC_DIAGONAL):
        newton = gb.NewtonInverseOperator(tolerance=1e-10, preconditioner=pc, linear_tolerance=1e-13, max_iterations=50)
        newton.bind(op)
        w = gb.DeviceArray(op.size)
        w.clear()
        rhs = gb.DeviceArray(op.size)
        rhs.clear()
        newton(rhs, w)
        info = newton.info()
        assert info["converged"] and info["failure"] == "Success", info
        assert info["iterations"] == io["iterations"]
        assert info["residual"] < 1e-10
        assert relmax(w.numpy(), wo) < 1e-9


@pytest.mark.gpu
def test_newton_line_search_matches_oracle(gb, orc):
    """r = u^3 - u from near the inflection point with weak diffusion: the
    Jacobian is indefinite (GMRES) and the line search halves overshooting
    steps, as in the oracle."""
    no = _no()
    cells, order, reaction = (2, 2, 2), 1, (-1.0, 1.0, 0.0)
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction, diffusion=1e-3)
    prob = orc.DGProblem(cells, order, diffusion=1e-3)
    P = no.NonlinearProblem(prob, reaction)
    w0 = prob.project(2, params=(0.58,))
    solve = lambda w, r, tol: (np.linalg.solve(P.jacobian_matrix(w), r), 1)
    wo, io = no.newton(P.apply, solve, np.zeros(op.size), w0, tolerance=1e-10, line_search=True)
    assert io["line_search_halvings"] > 0
    newton = gb.NewtonInverseOperator(tolerance=1e-10, line_search="simple", linear_method="gmres",
                                      linear_tolerance=1e-14, linear_restart=40, preconditioner=gb.PC_BLOCK_JACOBI,
                                      max_iterations=50)
    newton.bind(op)
    w = gb.DeviceArray.from_numpy(w0)
    rhs = gb.DeviceArray(op.size)
    rhs.clear()
    newton(rhs, w)
    info = newton.info()
    assert info["converged"], info
    assert info["iterations"] == io["iterations"]
    assert relmax(w.numpy(), wo) < 1e-8


@pytest.mark.gpu
def test_newton_eisenstat_walker_forcing_saves_linear_iterations(gb):
    cells, order, reaction = (6, 6, 6), 2, (0.0, 4.0, -2.0)
    op = gb.NonlinearDGOperator(cells, order, reaction=reaction)
    f = gb.project(cells, order, gb.FN_CONSTANT, params=(10.0,), scale_by_volume=True)
    res = {}
    for forcing in ("none", "eisenstatwalker"):
        # GMRES: right preconditioning, so its stopping test is the true
        # residual |J dw - r| <= eta |r| that the forcing term is meant for
        newton = gb.NewtonInverseOperator(tolerance=1e-9, forcing=forcing, linear_tolerance=1e-12,
                                          linear_method="gmres", linear_restart=50, max_iterations=50)
        newton.bind(op)
        w = gb.DeviceArray(op.size)
        w.clear()
        newton(f, w)
        res[forcing] = (newton.info(), w.numpy())
    for info, _ in res.values():
        assert info["converged"] and info["residual"] < 1e-9, info
    assert res["eisenstatwalker"][0]["linear_iterations"] < res["none"][0]["linear_iterations"]
    assert relmax(res["eisenstatwalker"][1], res["none"][1]) < 1e-7


@pytest.mark.gpu
def test_newton_on_a_linear_operator_is_one_linear_solve(gb, orc):
    cells, order = (3, 3, 3), 2
    op = gb.DGOperator(cells, order, mass=0.5)
    f = np.random.default_rng(5).uniform(-1, 1, op.size)
    newton = gb.NewtonInverseOperator(tolerance=1e-10, linear_tolerance=1e-12, max_iterations=50)
    newton.bind(op)
    w = gb.DeviceArray(op.size)
    w.clear()
    newton(gb.DeviceArray.from_numpy(f), w)
    info = newton.info()
    assert info["iterations"] == 0 and info["linear_iterations"] > 0 and info["converged"]
    prob = orc.DGProblem(cells, order, mass=0.5)
    assert np.linalg.norm(prob.apply(w.numpy()) - f) <= 1e-11 * np.linalg.norm(f) * 10


@pytest.mark.gpu
def test_nonlinear_pipelined_host_apply_is_bitwise_the_device_apply(gb):
    cells = (4, 3, 9)
    op = gb.NonlinearDGOperator(cells, 2, reaction=(0.1, 0.5, -0.2), periodic=(0, 0, 1))
    op.set_host_chunks(4)
    u = np.random.default_rng(6).uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    wh = np.empty(op.size)
    op.apply_host(u, wh)
    assert np.array_equal(wh.view(np.uint64), w.numpy().view(np.uint64))


@pytest.mark.gpu
def test_newton_stops_when_the_linear_solves_make_no_progress(gb):
    """Preconditioned CG with a linear tolerance so loose that <r, B r> <=
    eps^2 <b, b> holds at the start: dw = 0 twice, Newton ends as a linear
    solver failure instead of repeating the step."""
    cells, order = (4, 4, 4), 2
    op = gb.NonlinearDGOperator(cells, order, reaction=(0.0, 1.0, 0.0))
    f = gb.project(cells, order, gb.FN_CONSTANT, params=(1.0,), scale_by_volume=True)
    newton = gb.NewtonInverseOperator(tolerance=1e-12, linear_tolerance=0.999, preconditioner=gb.PC_BLOCK_JACOBI,
                                      max_iterations=1000)
    newton.bind(op)
    w = gb.DeviceArray(op.size)
    w.clear()
    newton(f, w)
    info = newton.info()
    assert not info["converged"] and info["failure"] == "LinearSolverFailed" and info["iterations"] < 1000


# ------------------------------------------------- run-time compiled reactions --
_USER = ("ipow<3>(u) + 0.5*exp(u) - sin(3.0*x)*y + 0.25*z*u",
         lambda u, x, y, z: u ** 3 + 0.5 * np.exp(u) - np.sin(3.0 * x) * y + 0.25 * z * u,
         lambda u, x, y, z: 3 * u ** 2 + 0.5 * np.exp(u) + 0.25 * z)


def test_user_reaction_source_compiles_for_sm103a():
    """The generated kernel compiles (nvcc, sm_103a cubin) for both precisions;
    expressions with other characters are refused."""
    import shutil
    if shutil.which("nvcc") is None and not __import__("os").path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not present")
    import gbfem
    import integrands
    for prec in (gbfem.F64, gbfem.F32):
        path = integrands.compile_reaction(_USER[0], prec, 2)
        assert path.endswith(".cubin") and __import__("os").path.getsize(path) > 0
    with pytest.raises(ValueError):
        integrands.reaction_source("u; system(1)", gbfem.F64, 2)
    src = integrands.reaction_source("u*u", gbfem.F32, 3, 4)
    assert "gbfem_user_reaction_f32_n4_q4" in src


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2, 3])
def test_user_reaction_apply_and_jacobian_match_oracle(gb, orc, order):
    import integrands
    no = _no()
    cells = (3, 2, 4)
    kw = dict(mass=0.3, velocity=(0.2, 0.0, -0.1), lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    op = integrands.UserNonlinearDGOperator(cells, order, _USER[0], **kw)
    assert op.nonlinear()
    P = no.NonlinearProblem(orc.DGProblem(cells, order, **kw), (_USER[1], _USER[2]))
    rng = np.random.default_rng(60 + order)
    u, d = rng.uniform(-1, 1, op.size), rng.uniform(-1, 1, op.size)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), P.apply(u)) < TOL64
    jac = op.jacobian(gb.DeviceArray.from_numpy(u))
    y = gb.DeviceArray(op.size)
    jac(gb.DeviceArray.from_numpy(d), y)
    assert relmax(y.numpy(), P.jacobian_apply(u, d)) < TOL64
    nl = op.nloc
    assert relmax(jac.block_diagonal(nl).numpy().reshape(-1, nl, nl), P.jacobian_blocks(u)) < TOL64


@pytest.mark.gpu
def test_user_reaction_newton_matches_oracle_newton(gb, orc):
    import integrands
    no = _no()
    cells, order = (3, 3, 3), 2
    expr = "ipow<3>(u) - 2.0*exp(u)*(1.0 + 0.5*x*y) + 0.0*z"
    r = lambda u, x, y, z: u ** 3 - 2.0 * np.exp(u) * (1.0 + 0.5 * x * y)
    dr = lambda u, x, y, z: 3 * u ** 2 - 2.0 * np.exp(u) * (1.0 + 0.5 * x * y)
    op = integrands.UserNonlinearDGOperator(cells, order, expr)
    P = no.NonlinearProblem(orc.DGProblem(cells, order), (r, dr))
    solve = lambda w, res, tol: (np.linalg.solve(P.jacobian_matrix(w), res), 1)
    wo, io = no.newton(P.apply, solve, np.zeros(op.size), np.zeros(op.size), tolerance=1e-10)
    newton = gb.NewtonInverseOperator(tolerance=1e-10, linear_tolerance=1e-13, max_iterations=50)
    newton.bind(op)
    w = gb.DeviceArray(op.size)
    w.clear()
    rhs = gb.DeviceArray(op.size)
    rhs.clear()
    newton(rhs, w)
    info = newton.info()
    assert info["converged"] and info["iterations"] == io["iterations"], (info, io)
    assert relmax(w.numpy(), wo) < 1e-9


@pytest.mark.gpu
def test_user_reaction_fp32(gb, orc):
    import integrands
    no = _no()
    cells, order = (3, 3, 2), 2
    op = integrands.UserNonlinearDGOperator(cells, order, _USER[0], precision=gb.F32)
    P = no.NonlinearProblem(orc.DGProblem(cells, order), (_USER[1], _USER[2]))
    u = np.random.default_rng(3).uniform(-1, 1, op.size).astype(np.float32)
    w = gb.DeviceArray(op.size, gb.F32)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), P.apply(u.astype(np.float64))) < 2e-5


def test_oracle_user_reaction_coordinates(orc):
    """r(u, x, y, z) = x + 2 y - z: the coefficient of phi_0 of R is |K| times
    that function at the cell centre (orthonormal basis, linear integrand)."""
    no = _no()
    cells = (2, 3, 2)
    prob = orc.DGProblem(cells, 1, lower=(0.0, -1.0, 0.5), upper=(1.0, 0.5, 1.5))
    P = no.NonlinearProblem(prob, (lambda u, x, y, z: x + 2 * y - z + 0 * u, lambda u, x, y, z: 0 * u))
    R = P.reaction(np.zeros(prob.ndofs)).reshape(-1, prob.nloc)
    h = (prob.upper - prob.lower) / prob.cells
    vol = float(np.prod(h))
    for c in range(prob.ncells):
        ix, iy, iz = c % 2, (c // 2) % 3, c // 6
        xc, yc, zc = prob.lower + (np.array([ix, iy, iz]) + 0.5) * h
        assert abs(R[c, 0] - vol * (xc + 2 * yc - zc)) < 1e-14


@pytest.mark.gpu
def test_projection_of_a_generated_expression(gb, orc):
    """integrands.project: exact for a polynomial in Q_p, and the same as the
    built-in projection for the Gaussian bump."""
    import integrands
    cells, order = (3, 2, 4), 2
    lower, upper = (0.0, -1.0, 0.5), (1.0, 0.5, 1.5)
    u = integrands.project(cells, order, "1.0 + 2.0*x - y + x*y*z + z*z", lower=lower, upper=upper).numpy()
    import vtkio
    vals = vtkio.evaluate_subcells(u, cells, order, level=1)
    h = [(upper[k] - lower[k]) / cells[k] for k in range(3)]
    zc = lower[2] + (np.arange(cells[2] * 2) + 0.5) * h[2] / 2
    yc = lower[1] + (np.arange(cells[1] * 2) + 0.5) * h[1] / 2
    xc = lower[0] + (np.arange(cells[0] * 2) + 0.5) * h[0] / 2
    X, Y, Z = xc[None, None, :], yc[None, :, None], zc[:, None, None]
    assert relmax(vals, 1.0 + 2.0 * X - Y + X * Y * Z + Z * Z) < 1e-13
    bump = integrands.project((4, 4, 4), 2, "exp(-((x-0.5)*(x-0.5) + (y-0.5)*(y-0.5) + (z-0.5)*(z-0.5))/(0.1*0.1))")
    ref = gb.project((4, 4, 4), 2, gb.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.1))
    assert relmax(bump.numpy(), ref.numpy()) < 1e-12
