"""General DG forms compiled at run time (integrands.Form, csrc/form_kernel.cuh):
the form oracle pinned to the DG oracle, the GPU kernels against the form
oracle (scalar and systems, FP64 and FP32), the dual-number Jacobian (apply,
blocks, diagonal, assembly) against differences of the residual, and Newton,
Scheme and RK3 over a generated form."""
import shutil

import numpy as np
import pytest

from conftest import relmax

PI = np.pi


def _sipg_linear(fo, eps, c, b):
    bv = np.array(b, dtype=np.float64)
    adv = (lambda x, u: bv[None, None, :] * u[:, :, None]) if any(b) else None
    ws = (lambda x, u, n: np.full(u.shape[0], abs(bv @ n))) if any(b) else None
    return fo.sipg(1, flux=lambda x, u, g: eps * g, source=lambda x, u, g: c * u, advection=adv, wavespeed=ws,
                   dirichlet=lambda x: np.zeros((x.shape[0], 1)))


def _linear_form(integrands, eps, c, b):
    adv = "for (int k = 0; k < 3; ++k) Fa[0][k] = u[0] * %r * (k == 0 ? %r : (k == 1 ? %r : %r));" % (1.0, *b)
    return integrands.Form(
        flux="for (int k = 0; k < 3; ++k) F[0][k] = %r * g[0][k];" % eps, source="s[0] = %r * u[0];" % c,
        advection=adv if any(b) else None,
        wavespeed="fabs(%r * n[0] + %r * n[1] + %r * n[2])" % tuple(b) if any(b) else None, dirichlet="")


# ---- the nonlinear scalar test form -------------------------------------------
# F = (1 + u^2) grad u + 0.3 u (g_y, -g_x, 0) (A non-symmetric), s = u^3 - sin(x) y,
# gD = x y + 0.5
_NL_FLUX = """const D a = 1.0 + u[0] * u[0];
F[0][0] = a * g[0][0] + 0.3 * u[0] * g[0][1];
F[0][1] = a * g[0][1] - 0.3 * u[0] * g[0][0];
F[0][2] = a * g[0][2];"""
_NL_SOURCE = "s[0] = u[0] * u[0] * u[0] - sin(x[0]) * x[1];"
_NL_DIRICHLET = "gD[0] = x[0] * x[1] + 0.5;"


def _nl_oracle(fo):
    def flux(x, u, g):
        a = 1.0 + u[:, 0] ** 2
        F = np.zeros(g.shape, dtype=np.result_type(u, g))
        F[:, 0, 0] = a * g[:, 0, 0] + 0.3 * u[:, 0] * g[:, 0, 1]
        F[:, 0, 1] = a * g[:, 0, 1] - 0.3 * u[:, 0] * g[:, 0, 0]
        F[:, 0, 2] = a * g[:, 0, 2]
        return F
    return fo.sipg(1, flux=flux, source=lambda x, u, g: u ** 3 - (np.sin(x[:, 0]) * x[:, 1])[:, None],
                   dirichlet=lambda x: (x[:, 0] * x[:, 1] + 0.5)[:, None])


# ---- a two-component system ---------------------------------------------------
# F0 = grad u0 + 0.2 u1 grad u1, F1 = (1 + u0^2) grad u1; s0 = u0 u1, s1 = -u0 + cos(z);
# convective flux of u1: b u1^2 / 2 (wave speed |b.n u1|); periodic in x, gD = (0, y)
_SYS_FLUX = """for (int k = 0; k < 3; ++k) {
  F[0][k] = g[0][k] + 0.2 * u[1] * g[1][k];
  F[1][k] = (1.0 + u[0] * u[0]) * g[1][k];
}"""
_SYS_SOURCE = "s[0] = u[0] * u[1]; s[1] = -u[0] + cos(x[2]);"
_B = (0.6, -0.3, 0.2)
_SYS_ADV = "for (int k = 0; k < 3; ++k) Fa[1][k] = 0.5 * u[1] * u[1] * (k == 0 ? %r : (k == 1 ? %r : %r));" % _B
_SYS_WS = "fabs((%r * n[0] + %r * n[1] + %r * n[2]) * u[1])" % _B
_SYS_DIRICHLET = "gD[0] = 0.0; gD[1] = x[1];"


def _sys_oracle(fo, smooth=False):
    """smooth: the constant wave speed 1 (no kink of max / fabs inside the
    difference quotients of the Jacobian test)."""
    bv = np.array(_B)

    def flux(x, u, g):
        F = np.zeros(g.shape, dtype=np.result_type(u, g))
        F[:, 0] = g[:, 0] + 0.2 * u[:, 1, None] * g[:, 1]
        F[:, 1] = (1.0 + u[:, 0, None] ** 2) * g[:, 1]
        return F

    def source(x, u, g):
        return np.stack([u[:, 0] * u[:, 1], -u[:, 0] + np.cos(x[:, 2])], axis=1)

    def adv(x, u):
        Fa = np.zeros(u.shape + (3,), dtype=u.dtype)
        Fa[:, 1] = 0.5 * u[:, 1, None] ** 2 * bv[None, :]
        return Fa

    return fo.sipg(2, flux=flux, source=source, advection=adv,
                   wavespeed=(lambda x, u, n: np.ones(u.shape[0])) if smooth else
                   (lambda x, u, n: np.abs((bv @ n) * u[:, 1])),
                   dirichlet=lambda x: np.stack([np.zeros(x.shape[0]), x[:, 1]], axis=1))


# ---- CPU: the oracle pin and the generator ----------------------------------------


@pytest.mark.parametrize("order,periodic,b", [(1, (0, 0, 0), (0.3, -0.2, 0.5)), (2, (1, 0, 1), (0.0, 0.4, -0.3)),
                                              (3, (0, 0, 0), (0.0, 0.0, 0.0))])
def test_form_oracle_equals_dg_oracle(orc, order, periodic, b):
    """The form oracle's interior-penalty form of F = eps grad u, s = c u,
    Fa = b u, gD = 0 is the SIPG / upwind / mass operator of oracle.cpp (itself
    pinned to the reference's tables and iterates)."""
    import form_oracle as fo
    cells, eps, c = (3, 2, 2), 0.7, 0.4
    lo, up = (0.1, -0.5, 0.0), (1.3, 0.5, 0.8)
    prob = orc.DGProblem(cells, order, diffusion=eps, mass=c, velocity=b, weak_dirichlet=True, periodic=periodic,
                         lower=lo, upper=up)
    I, S, Bd = _sipg_linear(fo, eps, c, b)
    spec = fo.FormSpec(cells, order, 1, I, S, Bd, penalty=eps * prob.penalty, periodic=periodic, lower=lo, upper=up)
    u = np.random.default_rng(order).uniform(-1, 1, prob.ndofs)
    assert relmax(fo.residual(spec, u), prob.apply(u)) < 1e-14


def test_form_oracle_transposed_flux_derivative():
    """A^T n of the symmetric face term by the complex step equals the analytic
    value for the non-symmetric test flux (A = (1+u^2) I + 0.3 u J)."""
    import form_oracle as fo
    _, skel, _ = _nl_oracle(fo)
    rng = np.random.default_rng(0)
    P = 7
    x = rng.uniform(0, 1, (P, 3))
    uL, uR = rng.uniform(-1, 1, (P, 1)), rng.uniform(-1, 1, (P, 1))
    gL, gR = rng.uniform(-1, 1, (P, 1, 3)), rng.uniform(-1, 1, (P, 1, 3))
    n = np.array([0.0, -1.0, 0.0])
    _, F = skel(x, n, 5.0, uL, gL, uR, gR)
    a = 1.0 + uL[:, 0] ** 2
    # A[j][k] = a delta_jk + 0.3 u (J)_{jk}, J = [[0, 1, 0], [-1, 0, 0], [0, 0, 0]]; A^T n
    J = np.array([[0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    ATn = a[:, None] * n[None, :] + 0.3 * uL[:, 0, None] * (J.T @ n)[None, :]
    expect = -0.5 * (uL[:, 0] - uR[:, 0])[:, None] * ATn
    assert np.max(np.abs(F[:, 0, :] - expect)) < 1e-14


def test_form_source_generation_and_compile(gb):
    import integrands
    f = integrands.Form(components=2, flux=_SYS_FLUX, source=_SYS_SOURCE, advection=_SYS_ADV, wavespeed=_SYS_WS,
                        dirichlet=_SYS_DIRICHLET)
    src = f.source_code(gb.F32, 1)
    assert "gbfem_form_f32_n2_q3_m2_val" in src and "gbfem_form_f32_n2_q3_m2_lin" in src
    with pytest.raises(ValueError):
        integrands.Form(flux="F[0][0] = 1; system(\"x\")\\")
    with pytest.raises(ValueError):
        integrands.Form(advection="Fa[0][0] = u[0];")  # no wave speed
    with pytest.raises(ValueError):
        integrands.Form(flux="F[0][0] = g[0][0];", interior="s[0] = u[0];")
    if shutil.which("nvcc") is None and not __import__("os").path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no nvcc")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        assert f.compile(gb.F32, 1, cache_dir=d).endswith(".cubin")
        raw = integrands.Form(interior="for (int k = 0; k < 3; ++k) F[0][k] = g[0][k];",
                              skeleton="s[0] = sigma * (uL[0] - uR[0]);", boundary="s[0] = sigma * u[0];")
        assert raw.compile(gb.F64, 2, cache_dir=d).endswith(".cubin")


# ---- GPU -----------------------------------------------------------------------------


def _rand(n, seed, scale=1.0):
    return scale * np.random.default_rng(seed).uniform(-1, 1, n)


@pytest.mark.gpu
@pytest.mark.parametrize("order,prec,periodic,b", [(1, 0, (0, 0, 0), (0.3, -0.2, 0.5)), (2, 0, (1, 0, 1), (0.0, 0.4, -0.3)),
                                                   (3, 0, (0, 0, 0), (0.2, 0.1, 0.0)), (2, 1, (0, 1, 0), (0.5, 0.0, 0.2))])
def test_linear_form_equals_dg_operator(gb, order, prec, periodic, b):
    """The generated SIPG / upwind / mass form is DGOperator's operator."""
    import integrands
    precision = gb.F64 if prec == 0 else gb.F32
    cells, eps, c = (3, 2, 4), 0.7, 0.4
    lo, up = (0.1, -0.5, 0.0), (1.3, 0.5, 0.8)
    beta = 10.0 * (order + 1) ** 2
    ref = gb.DGOperator(cells, order, precision=precision, diffusion=eps, mass=c, velocity=b, weak_dirichlet=True,
                        periodic=periodic, lower=lo, upper=up)
    op = integrands.FormOperator(_linear_form(integrands, eps, c, b), cells, order, precision=precision,
                                 penalty=eps * beta, periodic=periodic, lower=lo, upper=up)
    assert op.size == ref.size and op.nonlinear()
    u = gb.DeviceArray.from_numpy(_rand(op.size, order).astype(np.float64 if prec == 0 else np.float32))
    w1, w2 = gb.DeviceArray(op.size, precision), gb.DeviceArray(op.size, precision)
    op(u, w1)
    ref(u, w2)
    assert relmax(w1.numpy(), w2.numpy()) < (1e-12 if prec == 0 else 2e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("order,prec", [(1, 0), (2, 0), (3, 0), (2, 1)])
def test_nonlinear_form_against_oracle(gb, order, prec):
    import form_oracle as fo
    import integrands
    precision = gb.F64 if prec == 0 else gb.F32
    cells, lo, up = (3, 2, 2), (0.0, -0.4, 0.2), (1.2, 0.6, 1.0)
    form = integrands.Form(flux=_NL_FLUX, source=_NL_SOURCE, dirichlet=_NL_DIRICHLET)
    op = integrands.FormOperator(form, cells, order, precision=precision, lower=lo, upper=up)
    I, S, Bd = _nl_oracle(fo)
    spec = fo.FormSpec(cells, order, 1, I, S, Bd, lower=lo, upper=up)
    u = _rand(op.size, 7, 0.8)
    if prec:
        u = u.astype(np.float32).astype(np.float64)
    w = gb.DeviceArray(op.size, precision)
    op(gb.DeviceArray.from_numpy(u.astype(np.float64 if prec == 0 else np.float32)), w)
    assert relmax(w.numpy(), fo.residual(spec, u)) < (1e-12 if prec == 0 else 3e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("order,prec", [(1, 0), (2, 0), (1, 1)])
def test_system_form_against_oracle(gb, order, prec):
    import form_oracle as fo
    import integrands
    precision = gb.F64 if prec == 0 else gb.F32
    cells, periodic = (4, 2, 2), (1, 0, 0)
    form = integrands.Form(components=2, flux=_SYS_FLUX, source=_SYS_SOURCE, advection=_SYS_ADV,
                           wavespeed=_SYS_WS, dirichlet=_SYS_DIRICHLET)
    op = integrands.FormOperator(form, cells, order, precision=precision, periodic=periodic)
    assert op.size == 2 * (order + 1) ** 3 * 16
    I, S, Bd = _sys_oracle(fo)
    spec = fo.FormSpec(cells, order, 2, I, S, Bd, periodic=periodic)
    u = _rand(op.size, 11, 0.7)
    if prec:
        u = u.astype(np.float32).astype(np.float64)
    w = gb.DeviceArray(op.size, precision)
    op(gb.DeviceArray.from_numpy(u.astype(np.float64 if prec == 0 else np.float32)), w)
    assert relmax(w.numpy(), fo.residual(spec, u)) < (1e-12 if prec == 0 else 3e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("system", [False, True])
def test_form_jacobian(gb, system):
    """S'(u) du, the diagonal blocks, the diagonal and the assembled matrix of
    the dual-number linearisation against differences of the oracle's residual
    and against the Jacobian's own apply on unit vectors."""
    import form_oracle as fo
    import integrands
    if system:
        cells, order, periodic, M = (3, 2, 1), 1, (1, 0, 0), 2
        form = integrands.Form(components=2, flux=_SYS_FLUX, source=_SYS_SOURCE, advection=_SYS_ADV,
                               wavespeed="1.0", dirichlet=_SYS_DIRICHLET)
        I, S, Bd = _sys_oracle(fo, smooth=True)
    else:
        cells, order, periodic, M = (2, 2, 2), 1, (0, 0, 0), 1
        form = integrands.Form(flux=_NL_FLUX, source=_NL_SOURCE, dirichlet=_NL_DIRICHLET)
        I, S, Bd = _nl_oracle(fo)
    op = integrands.FormOperator(form, cells, order, periodic=periodic)
    spec = fo.FormSpec(cells, order, M, I, S, Bd, periodic=periodic)
    n, nloc = op.size, op.nloc
    u, du = _rand(n, 3, 0.8), _rand(n, 4)
    jac = op.jacobian(gb.DeviceArray.from_numpy(u))
    assert not jac.nonlinear()
    Jdu = gb.DeviceArray(n)
    jac(gb.DeviceArray.from_numpy(du), Jdu)
    assert relmax(Jdu.numpy(), fo.linearize(spec, u, du)) < 1e-9
    # the whole Jacobian, column by column, through the apply
    Jfull = np.zeros((n, n))
    col = gb.DeviceArray(n)
    for j in range(n):
        v = np.zeros(n)
        v[j] = 1.0
        jac(gb.DeviceArray.from_numpy(v), col)
        Jfull[:, j] = col.numpy()
    ncell = n // nloc
    blocks = jac.block_diagonal(nloc).numpy().reshape(ncell, nloc, nloc)
    for c in range(ncell):
        sl = slice(c * nloc, (c + 1) * nloc)
        assert np.max(np.abs(blocks[c] - Jfull[sl, sl])) < 1e-12 * np.max(np.abs(Jfull))
    assert np.max(np.abs(jac.diagonal().numpy() - np.diag(Jfull))) < 1e-12 * np.max(np.abs(Jfull))
    A = jac.assemble()
    y = gb.DeviceArray(n)
    A(gb.DeviceArray.from_numpy(du), y)
    assert relmax(y.numpy(), Jfull @ du) < 1e-12
    # the linearisation point is what jacobian() was given: a second point moves it
    op.jacobian(gb.DeviceArray.from_numpy(0.5 * u), jac)
    jac(gb.DeviceArray.from_numpy(du), Jdu)
    assert relmax(Jdu.numpy(), fo.linearize(spec, 0.5 * u, du)) < 1e-9


_PI = "3.141592653589793"
# -div((1 + u^2) grad u) = f for u* = sin(pi x) sin(pi y) sin(pi z), zero Dirichlet data
_MMS_SOURCE = ("const R px = %s * x[0], py = %s * x[1], pz = %s * x[2];\n"
               "const R us = sin(px) * sin(py) * sin(pz);\n"
               "const R gs = %s * %s * (cos(px) * cos(px) * sin(py) * sin(py) * sin(pz) * sin(pz)"
               " + sin(px) * sin(px) * cos(py) * cos(py) * sin(pz) * sin(pz)"
               " + sin(px) * sin(px) * sin(py) * sin(py) * cos(pz) * cos(pz));\n"
               "s[0] = -(3.0 * %s * %s * (1.0 + us * us) * us - 2.0 * us * gs);") % ((_PI,) * 7)


@pytest.mark.gpu
def test_newton_and_scheme_on_generated_form(gb):
    """Newton (GMRES, block Jacobi of the dual-number Jacobian) solves the
    quasilinear manufactured problem; the error against the projected exact
    solution falls at the order of the space; Scheme runs the same solve."""
    import integrands
    form = integrands.Form(flux="for (int k = 0; k < 3; ++k) F[0][k] = (1.0 + u[0] * u[0]) * g[0][k];",
                           source=_MMS_SOURCE, dirichlet="")
    order, errs = 2, []
    for N in (4, 8):
        op = integrands.FormOperator(form, (N, N, N), order)
        newton = gb.NewtonInverseOperator(tolerance=1e-10, linear_method="gmres", linear_tolerance=1e-12,
                                          preconditioner=gb.PC_BLOCK_JACOBI)
        newton.bind(op)
        w = gb.DeviceArray(op.size)
        w.clear()
        rhs = gb.DeviceArray(op.size)
        rhs.clear()
        newton(rhs, w)
        info = newton.info()
        assert info["converged"] and 2 <= info["iterations"] <= 8, info
        exact = integrands.project((N, N, N), order, "sin(%s*x)*sin(%s*y)*sin(%s*z)" % ((_PI,) * 3))
        errs.append(np.sqrt(np.sum((w.numpy() - exact.numpy()) ** 2) / N ** 3))
        if N == 4:
            scheme = gb.Scheme(op, parameters={"nonlinear.tolerance": 1e-10, "linear.method": "gmres",
                                               "linear.tolerance": 1e-12,
                                               "linear.preconditioning.method": "blockjacobi"})
            z = scheme.space.zero
            assert scheme.solve(target=z)["converged"]
            assert relmax(z.numpy(), w.numpy()) < 1e-8
            # Newton on each Jacobian assembled into the block-sparse matrix: the same steps
            na = gb.NewtonInverseOperator(tolerance=1e-10, linear_method="gmres", linear_tolerance=1e-12,
                                          preconditioner=gb.PC_BLOCK_JACOBI, assembled=True)
            na.bind(op)
            wa = gb.DeviceArray(op.size)
            wa.clear()
            na(rhs, wa)
            assert na.info()["converged"] and na.info()["iterations"] == info["iterations"]
            assert relmax(wa.numpy(), w.numpy()) < 1e-8
    assert errs[1] < errs[0] / 5.0, errs


@pytest.mark.gpu
def test_rk3_steps_a_generated_form(gb):
    """RK3 over the generated linear advection form equals RK3 over DGOperator."""
    import integrands
    b = (0.8, -0.4, 0.3)
    cells, order = (4, 4, 4), 2
    form = integrands.Form(advection="for (int k = 0; k < 3; ++k) Fa[0][k] = u[0] * (k == 0 ? %r : (k == 1 ? %r : %r));" % b,
                           wavespeed="fabs(%r * n[0] + %r * n[1] + %r * n[2])" % b)
    op = integrands.FormOperator(form, cells, order, periodic=(1, 1, 1))
    ref = gb.DGOperator(cells, order, diffusion=0.0, velocity=b, periodic=(1, 1, 1), weak_dirichlet=False)
    u0 = _rand(op.size, 5)
    ua, ub = gb.DeviceArray.from_numpy(u0), gb.DeviceArray.from_numpy(u0)
    ra, rb = gb.RK3(op), gb.RK3(ref)
    for _ in range(5):
        ra.step(ua, 1e-3)
        rb.step(ub, 1e-3)
    assert relmax(ua.numpy(), ub.numpy()) < 1e-12


# ---- the UFL-shaped front end ------------------------------------------------------


def _ufl_scalar():
    from ufl_forms import (TestFunction, TrialFunction, SpatialCoordinate, grad, inner, dx, sin, to_form,
                           as_vector)
    u, v, x = TrialFunction(1), TestFunction(1), SpatialCoordinate()
    gu = grad(u)[0, :]
    a = (1 + u[0] ** 2)
    F = as_vector([a * gu[0] + 0.3 * u[0] * gu[1], a * gu[1] - 0.3 * u[0] * gu[0], a * gu[2]])
    form = inner(F, grad(v)[0, :]) * dx + (u[0] ** 3 - sin(x[0]) * x[1]) * v[0] * dx
    return to_form(form, dirichlet=[x[0] * x[1] + 0.5])


def _ufl_system():
    from ufl_forms import (TestFunction, TrialFunction, SpatialCoordinate, FacetNormal, grad, inner, dx, cos,
                           to_form)
    u, v, x, n = TrialFunction(2), TestFunction(2), SpatialCoordinate(), FacetNormal()
    F0 = grad(u)[0, :] + 0.2 * u[1] * grad(u)[1, :]
    F1 = (1.0 + u[0] ** 2) * grad(u)[1, :]
    form = (inner(F0, grad(v)[0, :]) + inner(F1, grad(v)[1, :]) + u[0] * u[1] * v[0]
            + (-u[0] + cos(x[2])) * v[1]) * dx
    b = _B
    bn = b[0] * n[0] + b[1] * n[1] + b[2] * n[2]
    return to_form(form, components=2, advection=[[0.0, 0.0, 0.0], [0.5 * u[1] ** 2 * bk for bk in b]],
                   wavespeed=abs(bn * u[1]), dirichlet=[0.0, x[1]])


def test_ufl_front_end_lowers_and_compiles(gb):
    import ufl_forms as U
    f = _ufl_scalar()
    assert "F[0][0]" in f.pieces["flux"] and "s[0]" in f.pieces["source"] and "gD[0]" in f.pieces["dirichlet"]
    g = _ufl_system()
    assert g.components == 2 and "Fa[1][2]" in g.pieces["advection"] and "fabs" in g.pieces["wavespeed"]
    u, v = U.TrialFunction(1), U.TestFunction(1)
    with pytest.raises(ValueError):
        (v[0] * v[0]) * U.dx  # not linear in v
    with pytest.raises(ValueError):
        (u[0] * v[0]) * U.dS  # facet integrals need restrictions (tests/test_ufl_faces.py)
    with pytest.raises(TypeError):
        U.grad(3.0)
    if shutil.which("nvcc") is None and not __import__("os").path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no nvcc")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        assert g.compile(gb.F64, 1, cache_dir=d).endswith(".cubin")


@pytest.mark.gpu
@pytest.mark.parametrize("system", [False, True])
def test_ufl_forms_against_oracle(gb, system):
    """The UFL-written forms equal the oracle of the same forms (and so the
    hand-written pieces of the tests above)."""
    import form_oracle as fo
    import integrands
    if system:
        cells, order, periodic, M, form, orc = (4, 2, 2), 2, (1, 0, 0), 2, _ufl_system(), _sys_oracle(fo)
    else:
        cells, order, periodic, M, form, orc = (3, 2, 2), 2, (0, 0, 0), 1, _ufl_scalar(), _nl_oracle(fo)
    lo, up = ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)) if system else ((0.0, -0.4, 0.2), (1.2, 0.6, 1.0))
    op = integrands.FormOperator(form, cells, order, periodic=periodic, lower=lo, upper=up)
    spec = fo.FormSpec(cells, order, M, *orc, periodic=periodic, lower=lo, upper=up)
    u = _rand(op.size, 21, 0.7)
    w = gb.DeviceArray(op.size)
    op(gb.DeviceArray.from_numpy(u), w)
    assert relmax(w.numpy(), fo.residual(spec, u)) < 1e-12
    du = _rand(op.size, 22)
    if not system:  # smooth: the Jacobian against differences of the oracle
        jac = op.jacobian(gb.DeviceArray.from_numpy(u))
        y = gb.DeviceArray(op.size)
        jac(gb.DeviceArray.from_numpy(du), y)
        assert relmax(y.numpy(), fo.linearize(spec, u, du)) < 1e-9


@pytest.mark.gpu
def test_form_operator_rejects_mismatched_cubins_and_arguments(gb):
    """A cubin compiled for another order (or component count) is refused
    with an error naming the missing kernels; 5 components and a kappa are
    refused; nothing is created."""
    import ctypes as C
    import integrands
    L = gb.lib()
    L.gbfem_form_operator_create.argtypes = [C.POINTER(gb.DgDesc), C.c_int, C.c_char_p, C.POINTER(C.c_void_p)]
    cub = integrands.Form(flux="for (int k = 0; k < 3; ++k) F[0][k] = g[0][k];").compile(gb.F64, 1)
    d = gb.DgDesc()
    d.grid = gb.grid_desc((2, 2, 2))
    d.order, d.quad_points, d.precision, d.penalty = 2, 4, gb.F64, 90.0
    for comps in (1, 2, 5):  # order 2 against an order-1 cubin; 2 components; 5 components
        h = C.c_void_p()
        assert L.gbfem_form_operator_create(C.byref(d), comps, cub.encode(), C.byref(h)) != 0
        assert not h.value
    d.order, d.quad_points = 1, 3
    h = C.c_void_p()
    assert L.gbfem_form_operator_create(C.byref(d), 1, b"/nonexistent/form.cubin", C.byref(h)) != 0
    assert L.gbfem_form_operator_create(C.byref(d), 1, cub.encode(), C.byref(h)) == 0 and h.value
    L.gbfem_operator_destroy(h)
    # the refused loads leave no error behind for the next launch
    op = gb.DGOperator((2, 2, 2), 1)
    x, y = gb.DeviceArray.from_numpy(np.ones(op.size)), gb.DeviceArray(op.size)
    op(x, y)


@pytest.mark.parametrize("order", [1, 2])
def test_form_oracle_natural_boundary_equals_dg_oracle(orc, order):
    """Without Dirichlet data the interior-penalty form has no boundary terms
    for a pure diffusion: the DG oracle's do-nothing boundary."""
    import form_oracle as fo
    cells, eps, c = (3, 2, 2), 1.3, 0.2
    prob = orc.DGProblem(cells, order, diffusion=eps, mass=c, weak_dirichlet=False)
    I, S, Bd = fo.sipg(1, flux=lambda x, u, g: eps * g, source=lambda x, u, g: c * u)
    spec = fo.FormSpec(cells, order, 1, I, S, Bd, penalty=eps * prob.penalty)
    u = np.random.default_rng(7 + order).uniform(-1, 1, prob.ndofs)
    assert relmax(fo.residual(spec, u), prob.apply(u)) < 1e-14


def test_form_oracle_linearisation_is_consistent():
    """The oracle's Richardson-difference linearisation is linear in the
    direction and matches a small central difference (a check of the
    checker used by the GPU Jacobian tests)."""
    import form_oracle as fo
    I, S, Bd = _nl_oracle(fo)
    spec = fo.FormSpec((2, 2, 1), 1, 1, I, S, Bd)
    rng = np.random.default_rng(3)
    u, a, b = (rng.uniform(-0.5, 0.5, spec.ndofs) for _ in range(3))
    ja, jb, jab = fo.linearize(spec, u, a), fo.linearize(spec, u, b), fo.linearize(spec, u, 2.0 * a - b)
    assert relmax(jab, 2.0 * ja - jb) < 1e-9
    h = 1e-6
    cd = (fo.residual(spec, u + h * a) - fo.residual(spec, u - h * a)) / (2 * h)
    assert relmax(ja, cd) < 1e-7


@pytest.mark.parametrize("components,order,prec", [(3, 3, 0), (4, 1, 1), (1, 4, 1), (2, 4, 0)])
def test_form_kernels_compile_for_more_shapes(gb, components, order, prec):
    """Kernel shapes beyond those the GPU tests run: 3 and 4 components,
    order 4 (q = 6), FP32 duals; each stays within the shared memory of one
    CTA (form_smem_bytes)."""
    import integrands
    if shutil.which("nvcc") is None and not __import__("os").path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("no nvcc")
    M = components
    flux = "for (int m = 0; m < %d; ++m) for (int k = 0; k < 3; ++k) F[m][k] = (1.0 + u[0] * u[0]) * g[m][k];" % M
    src = "for (int m = 0; m < %d; ++m) s[m] = u[m] * u[(m + 1) %% %d] - sin(x[m %% 3]);" % (M, M)
    adv = "for (int k = 0; k < 3; ++k) Fa[0][k] = 0.5 * u[0] * u[0];"
    form = integrands.Form(components=M, flux=flux, source=src, advection=adv,
                           wavespeed="fabs(u[0] * (n[0] + n[1] + n[2]))", dirichlet="gD[0] = x[0];")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        assert form.compile(gb.F64 if prec == 0 else gb.F32, order, cache_dir=d).endswith(".cubin")
    q, n = order + 2, order + 1
    cpb = 1 if q ** 3 * M >= 128 else (2 if 2 * q ** 3 * M >= 128 else 4)
    vol = cpb * M * (q * n * n + q * q * n + 4 * q ** 3)
    face = cpb * M * 8 * (n * n + q * n + 3 * q * q)
    rb = 8 if prec == 0 else 4
    smem = ((7 * 5 + 49 + 7 + 20) * rb + 15) // 16 * 16 + (2 * cpb * M * n ** 3 + max(vol, face)) * 2 * rb
    assert smem <= 227 * 1024
