"""Facet integrals in the UFL-shaped front end (dune-fem_gb300/ufl_forms.py).

The reference's advection-diffusion demo writes its SIPG / upwind form in
UFL with interior-facet (dS) and boundary (ds) terms
(pydemo/advectiondiffusion.py:33-55).  The same form written with this
package's UFL notation -- restrictions, jump, avg, the facet normal and the
facet size -- is lowered to the raw interior / skeleton / boundary bodies of
integrands.Form.  On the CPU the lowered integrands, evaluated by a small
tree walker here, go through the form oracle and must reproduce the DG
oracle's operator (itself pinned to dune-fem's DGEllipticOperator); on the
GPU the compiled form must equal DGOperator.
"""
import numpy as np
import pytest

from conftest import relmax

EPS, MASS, VEL = 0.7, 0.4, (1.0, 0.5, 0.25)


def demo_form(order, eps=EPS, c=MASS, b=VEL):
    """SIPG + upwind + mass with weak homogeneous Dirichlet data, in the
    demo's shape: penalty beta / h with h = avg(CellVolume) / FacetArea."""
    import ufl_forms as U
    u, v, x, n = U.TrialFunction(1), U.TestFunction(1), U.SpatialCoordinate(), U.FacetNormal()
    h = U.FacetSize()
    beta = 10.0 * (order + 1) ** 2
    bv = U.as_vector(list(b))
    gu, gv = U.grad(u)[0, :], U.grad(v)[0, :]
    bn = U.inner(bv, n.vector())
    hatb = (bn + abs(bn)) / 2.0
    a = (eps * U.inner(gu, gv) - u[0] * U.inner(bv, gv) + c * u[0] * v[0]) * U.dx
    a = a + (eps * beta / h * U.jump(u[0]) * U.jump(v[0])
             - eps * U.inner(U.avg(gu), n("+")) * U.jump(v[0])
             - eps * U.jump(u[0]) * U.inner(U.avg(gv), n("+"))) * U.dS
    a = a + U.jump(hatb * u[0]) * U.jump(v[0]) * U.dS
    a = a + (eps * beta / h * u[0] * v[0] - eps * U.inner(gu, n.vector()) * v[0]
             - eps * u[0] * U.inner(gv, n.vector())) * U.ds
    a = a + hatb * u[0] * v[0] * U.ds
    return a


# ---- a numpy evaluation of the lowered expression trees ------------------------------

def _ev(e, env):
    import ufl_forms as U
    if isinstance(e, U.Num):
        return e.v
    if isinstance(e, U.Leaf):
        return env[e.text]
    if isinstance(e, U.Op):
        a = [_ev(t, env) for t in e.args]
        if e.op in "+-*/" and len(a) == 2:
            return {"+": np.add, "-": np.subtract, "*": np.multiply, "/": np.divide}[e.op](a[0], a[1])
        if e.op == "-":
            return -a[0]
        if e.op.startswith("ipow"):
            return a[0] ** int(e.op[4:])
        return {"fabs": np.abs, "max": np.maximum, "min": np.minimum, "pow": np.power}.get(
            e.op, getattr(np, e.op, None))(*a)
    if isinstance(e, U.Cond):
        return {"<": np.less, ">": np.greater, "<=": np.less_equal, ">=": np.greater_equal}[e.op](
            _ev(e.a, env), _ev(e.b, env))
    if isinstance(e, U.Conditional):
        return np.where(_ev(e.c, env), _ev(e.a, env), _ev(e.b, env))
    raise TypeError(e)


def _integrand(part, side, M, env_of):
    def f(*args):
        env, P = env_of(*args)
        s, F = np.zeros((P, M)), np.zeros((P, M, 3))
        for key, c in part.terms.items():
            val = np.broadcast_to(_ev(c, env), (P,))
            if key[0] == "v" + side:
                s[:, key[1]] += val
            elif key[0] == "g" + side:
                F[:, key[1], key[2]] += val
        return s, F
    return f


def _fields(prefix, u, g):
    env = {}
    for m in range(u.shape[1]):
        env["%s[%d]" % (prefix, m)] = u[:, m]
        for k in range(3):
            env["%s[%d][%d]" % ("g" + prefix[1:], m, k)] = g[:, m, k]
    return env


def oracle_callables(a, M=1):
    def interior_env(x, u, g):
        env = {"x[%d]" % k: x[:, k] for k in range(3)}
        env.update(_fields("u", u, g))
        return env, x.shape[0]

    def skeleton_env(x, n, sigma, uL, gL, uR, gR):
        env = {"x[%d]" % k: x[:, k] for k in range(3)}
        env.update({"n[%d]" % k: n[k] for k in range(3)})
        env["(1.0 / sigma)"] = 1.0 / sigma
        env.update(_fields("uL", uL, gL))
        env.update(_fields("uR", uR, gR))
        return env, x.shape[0]

    def boundary_env(x, n, sigma, u, g):
        env = {"x[%d]" % k: x[:, k] for k in range(3)}
        env.update({"n[%d]" % k: n[k] for k in range(3)})
        env["(1.0 / sigma)"] = 1.0 / sigma
        env.update(_fields("u", u, g))
        return env, x.shape[0]

    p = a.parts
    return (_integrand(p["dx"], "", M, interior_env), _integrand(p["dS"], "+", M, skeleton_env),
            _integrand(p["ds"], "", M, boundary_env))


# ---- CPU ----------------------------------------------------------------------------------


@pytest.mark.parametrize("order,periodic", [(1, (0, 0, 0)), (2, (1, 0, 1)), (3, (0, 1, 0))])
def test_demo_form_in_ufl_equals_the_dg_oracle(orc, order, periodic):
    import form_oracle as fo
    cells = (3, 2, 2)
    lo, up = (0.1, -0.5, 0.0), (1.3, 0.5, 0.8)
    a = demo_form(order)
    I, S, B = oracle_callables(a)
    spec = fo.FormSpec(cells, order, 1, I, S, B, penalty=1.0, periodic=periodic, lower=lo, upper=up)
    prob = orc.DGProblem(cells, order, diffusion=EPS, mass=MASS, velocity=VEL, weak_dirichlet=True,
                         periodic=periodic, lower=lo, upper=up)
    u = np.random.default_rng(order).uniform(-1, 1, prob.ndofs)
    assert relmax(fo.residual(spec, u), prob.apply(u)) < 1e-13


def test_two_component_facet_form_is_two_sipg_operators(orc, gb, tmp_path):
    """Components 0 and 1 with their own diffusion, written with dS / ds
    terms on both: the residual of the interleaved dofs (cell M n^3 + i M + m)
    is the DG oracle's operator on each component."""
    import form_oracle as fo
    import ufl_forms as U
    cells, order, eps = (3, 2, 2), 2, (0.7, 1.9)
    u, v, n, h = U.TrialFunction(2), U.TestFunction(2), U.FacetNormal(), U.FacetSize()
    beta = 10.0 * (order + 1) ** 2
    a = None
    for m in range(2):
        gu, gv = U.grad(u)[m, :], U.grad(v)[m, :]
        t = eps[m] * U.inner(gu, gv) * U.dx
        t = t + (eps[m] * beta / h * U.jump(u[m]) * U.jump(v[m]) - eps[m] * U.inner(U.avg(gu), n("+")) * U.jump(v[m])
                 - eps[m] * U.jump(u[m]) * U.inner(U.avg(gv), n("+"))) * U.dS
        t = t + (eps[m] * beta / h * u[m] * v[m] - eps[m] * U.inner(gu, n.vector()) * v[m]
                 - eps[m] * u[m] * U.inner(gv, n.vector())) * U.ds
        a = t if a is None else a + t
    I, S, B = oracle_callables(a, M=2)
    spec = fo.FormSpec(cells, order, 2, I, S, B, penalty=1.0)
    nl = (order + 1) ** 3
    ncell = int(np.prod(cells))
    w = np.random.default_rng(5).uniform(-1, 1, (ncell, nl, 2))
    res = fo.residual(spec, w.reshape(-1)).reshape(ncell, nl, 2)
    for m in range(2):
        prob = orc.DGProblem(cells, order, diffusion=eps[m], weak_dirichlet=True)
        assert relmax(res[:, :, m].ravel(), prob.apply(np.ascontiguousarray(w[:, :, m]).ravel())) < 1e-13
    form = U.to_form(a, components=2)
    assert "s[1]" in form.pieces["skeleton"] and "uR[1]" in form.pieces["skeleton"]
    assert form.compile(gb.F64, order, cache_dir=str(tmp_path)).endswith(".cubin")


def test_demo_mesh_quantities_are_the_facet_size():
    """The demo's he = avg(CellVolume)/FacetArea and hbnd = CellVolume/FacetArea
    lower to the facet size: the same form source as with FacetSize()."""
    import ufl_forms as U
    space = U.dglegendre((3, 2, 2), 2)
    u, v, n = U.TrialFunction(1), U.TestFunction(1), U.FacetNormal()
    he = U.avg(U.CellVolume(space)) / U.FacetArea(space)
    hbnd = U.CellVolume(space) / U.FacetArea(space)
    h = U.FacetSize()

    def form(hi, hb):
        a = U.inner(U.grad(u)[0, :], U.grad(v)[0, :]) * U.dx
        a = a + 90.0 / hi * U.jump(u[0]) * U.jump(v[0]) * U.dS + 90.0 / hb * u[0] * v[0] * U.ds
        return U.to_form(a)

    assert form(he, hbnd).source_code(0, 2) == form(h, h).source_code(0, 2)
    with pytest.raises(ValueError):
        U.FacetArea(space) / U.CellVolume(space)


def test_lowering_and_errors(gb, tmp_path):
    import integrands
    import ufl_forms as U
    form = U.to_form(demo_form(2))
    assert form.raw and form.unit_penalty
    assert "uR[0]" in form.pieces["skeleton"] and "(1.0 / sigma)" in form.pieces["boundary"]
    assert "uL" not in form.pieces["interior"]
    assert form.compile(gb.F64, 2, cache_dir=str(tmp_path)).endswith(".cubin")
    u, v, n = U.TrialFunction(1), U.TestFunction(1), U.FacetNormal()
    with pytest.raises(ValueError):
        (u[0] * v[0]) * U.dS  # unrestricted in dS
    with pytest.raises(ValueError):
        (u[0]("+") * v[0]) * U.dS  # unrestricted test function in dS
    with pytest.raises(ValueError):
        (u[0]("+") * v[0]) * U.ds  # restriction in ds
    with pytest.raises(ValueError):
        (u[0] * v[0] * n[0]) * U.dx  # normal in dx
    with pytest.raises(ValueError):
        u[0]("+")("-")
    with pytest.raises(ValueError):
        U.to_form(demo_form(1), dirichlet=[0.0])  # face terms are in the form
    with pytest.raises(ValueError):
        integrands.FormOperator(form, (2, 2, 2), 2, penalty=90.0)


# ---- GPU ----------------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("order,periodic", [(1, (0, 0, 0)), (2, (1, 0, 1)), (3, (0, 1, 0))])
def test_demo_form_in_ufl_equals_dg_operator_on_gpu(gb, order, periodic):
    """The demo's form written in UFL notation, compiled at run time, is
    DGOperator's SIPG / upwind / mass operator."""
    import integrands
    import ufl_forms as U
    cells = (3, 2, 4)
    lo, up = (0.1, -0.5, 0.0), (1.3, 0.5, 0.8)
    op = integrands.FormOperator(U.to_form(demo_form(order)), cells, order, periodic=periodic, lower=lo, upper=up)
    ref = gb.DGOperator(cells, order, diffusion=EPS, mass=MASS, velocity=VEL, weak_dirichlet=True,
                        periodic=periodic, lower=lo, upper=up)
    u = gb.DeviceArray.from_numpy(np.random.default_rng(order).uniform(-1, 1, op.size))
    w1, w2 = gb.DeviceArray(op.size), gb.DeviceArray(op.size)
    op(u, w1)
    ref(u, w2)
    assert relmax(w1.numpy(), w2.numpy()) < 1e-12


# ---- derivatives of coefficient expressions ------------------------------------------


def test_grad_and_div_of_expressions_match_differences():
    """grad(e) and div(E) of expressions in x and u are the chain rule: against
    central differences of the evaluated trees at random points."""
    import ufl_forms as U
    x, u = U.SpatialCoordinate(), U.TrialFunction(1)
    e = U.sin(x[0] * x[1]) + x[2] ** 3 * U.exp(0.5 * u[0]) - U.atan(x[1] / (1 + x[0] ** 2)) \
        + U.sqrt(2 + U.cos(x[2])) * U.tanh(u[0] * x[0]) + abs(x[0] - 0.4) * U.log(3 + x[1])
    E = U.as_vector([x[1] * U.exp(-x[0]), U.sinh(x[1] * x[2]), U.max_value(x[0], x[2]) * x[2] ** 2])
    rng = np.random.default_rng(0)
    P = 40
    X = rng.uniform(0.05, 0.95, (P, 3))
    Uv = rng.uniform(-1, 1, (P, 1))
    G = rng.uniform(-1, 1, (P, 1, 3))

    def env(X, Uv, G):
        d = {"x[%d]" % k: X[:, k] for k in range(3)}
        d["u[0]"] = Uv[:, 0]
        d.update({"g[0][%d]" % k: G[:, 0, k] for k in range(3)})
        return d

    g = U.grad(e, components=1)
    h = 1e-6
    for k in range(3):
        # the total derivative along u(x) with du/dx_k = G[:, 0, k]
        Xp, Xm = X.copy(), X.copy()
        Xp[:, k] += h
        Xm[:, k] -= h
        fd = (_ev(e, env(Xp, Uv + h * G[:, :, k], G)) - _ev(e, env(Xm, Uv - h * G[:, :, k], G))) / (2 * h)
        assert np.max(np.abs(_ev(g[k], env(X, Uv, G)) - fd)) < 1e-7
    d = U.div(E)
    fd = 0.0
    for k in range(3):
        Xp, Xm = X.copy(), X.copy()
        Xp[:, k] += h
        Xm[:, k] -= h
        fd = fd + (_ev(E[k], env(Xp, Uv, G)) - _ev(E[k], env(Xm, Uv, G))) / (2 * h)
    assert np.max(np.abs(_ev(d, env(X, Uv, G)) - fd)) < 1e-7
    with pytest.raises(ValueError):
        U.grad(U.grad(u)[0, 0] * x[0])  # second derivatives of u
    with pytest.raises(TypeError):
        U.div(U.as_vector([x[0], x[1]]))


def test_demo_manufactured_right_hand_side_lowers_and_compiles(gb, tmp_path):
    """The demo's right-hand side -div(eps grad(exact) - b exact) v dx and its
    Neumann data eps grad(exact).n v ds, written with grad / div of the
    exact solution, lower to a form that compiles for sm_103a; the generated
    source term at a point equals the analytic one."""
    import ufl_forms as U
    x, v, n = U.SpatialCoordinate(), U.TestFunction(1), U.FacetNormal()
    eps, b = 0.1, U.as_vector([1.0, 0.0, 0.0])
    exact = U.sin(x[0] * x[1])
    rhs = -U.div(eps * U.grad(exact) - b * exact) * v[0] * U.dx + eps * U.inner(U.grad(exact), n.vector()) * v[0] * U.ds
    X = np.array([[0.3, 0.7, 0.2]])
    s = _ev(rhs.parts["dx"].terms[("v", 0)], {"x[%d]" % k: X[:, k] for k in range(3)})
    xx, yy = 0.3, 0.7
    lap = -(yy ** 2 + xx ** 2) * np.sin(xx * yy)
    expect = -(eps * lap - yy * np.cos(xx * yy))
    assert abs(float(np.ravel(s)[0]) - expect) < 1e-14
    form = U.to_form(rhs)
    assert form.compile(gb.F64, 1, cache_dir=str(tmp_path)).endswith(".cubin")
